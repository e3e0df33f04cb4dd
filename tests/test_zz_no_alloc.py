"""lbswim_spread_forces_noalloc: the allocation-free spreading entry point.

Callers that cannot allocate device memory (plug-in code inside a host
application that owns all device memory through its own allocator, real-time
loops that cannot afford an allocation's implicit synchronisation) pass their
own device buffers; the scratch is the library's static device array.  Its result must
equal that of lbswim_swimmers_add_forces on the same swimmers, on two calls in
a row (the second call finds the first call's leftovers in the scratch).
This file is collected last so that a failure here stops a run only after
every other test has run.
"""
import ctypes as C

import numpy as np
import pytest

import oracle as O
from gpu_harness import build_gpu
from helpers import TOL_F64, rel_l2_maxnorm

pytestmark = pytest.mark.gpu


def _dev(torch, a):
    return torch.tensor(np.ascontiguousarray(a, dtype=np.float64), device="cuda")


def test_noalloc_spread_matches_add_forces_twice():
    torch = pytest.importorskip("torch")
    from lbswim import _lib
    shape = (24, 20, 28)
    N = int(np.prod(shape))
    case = O.random_case(shape, 500, 0, seed=91, P=2e-3, l=0.4)
    lat, sw, _, _ = build_gpu(case, "f64")
    lat.ZeroForce()
    sw.AddForces(lat)
    lat.force.D2H()
    expected = lat.force.data.reshape(3, N).copy()
    assert np.abs(expected).max() > 0

    s = case["swimmers"]
    r = _dev(torch, s["r"])
    n = _dev(torch, s["nvec"])
    force = torch.empty(3 * N, dtype=torch.float64, device="cuda")
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    for call in range(2):
        force.fill_(123.0)  # overwrite mode must replace whatever is there
        rc = _lib.lib.lbswim_spread_forces_noalloc(
            C.c_void_p(r.data_ptr()), C.c_void_p(n.data_ptr()), s["n"], s["P"], s["l"],
            shape[0], shape[1], shape[2], C.c_void_p(force.data_ptr()), 0, stream)
        _lib.check(rc)
        torch.cuda.synchronize()
        got = force.cpu().numpy().reshape(3, N)
        assert rel_l2_maxnorm(got, expected) <= TOL_F64, call
        assert np.abs(got - expected).max() <= TOL_F64 * np.abs(expected).max(), call

    # accumulate mode adds the same spread on top
    rc = _lib.lib.lbswim_spread_forces_noalloc(
        C.c_void_p(r.data_ptr()), C.c_void_p(n.data_ptr()), s["n"], s["P"], s["l"],
        shape[0], shape[1], shape[2], C.c_void_p(force.data_ptr()), 1, stream)
    _lib.check(rc)
    torch.cuda.synchronize()
    assert rel_l2_maxnorm(force.cpu().numpy().reshape(3, N), 2 * expected) <= TOL_F64


def test_noalloc_spread_rejects_sizes_beyond_its_limit():
    torch = pytest.importorskip("torch")
    from lbswim import _lib
    force = torch.zeros(3 * 8 * 8 * 8, dtype=torch.float64, device="cuda")
    r = torch.zeros(3 * 16385, dtype=torch.float64, device="cuda")
    rc = _lib.lib.lbswim_spread_forces_noalloc(
        C.c_void_p(r.data_ptr()), C.c_void_p(r.data_ptr()), 16385, 1e-3, 0.5, 8, 8, 8,
        C.c_void_p(force.data_ptr()), 0, None)
    assert rc == -1 and b"limit" in _lib.lib.lbswim_last_error()
    rc = _lib.lib.lbswim_spread_forces_noalloc(
        C.c_void_p(r.data_ptr()), C.c_void_p(r.data_ptr()), 1, 1e-3, 0.5, 260, 260, 260,
        C.c_void_p(force.data_ptr()), 0, None)
    assert rc == -1 and b"limit" in _lib.lib.lbswim_last_error()
    # a swimmer count that would wrap when doubled
    rc = _lib.lib.lbswim_spread_forces_noalloc(
        C.c_void_p(r.data_ptr()), C.c_void_p(r.data_ptr()), 2 ** 31 - 1, 1e-3, 0.5, 8, 8, 8,
        C.c_void_p(force.data_ptr()), 0, None)
    assert rc == -1 and b"limit" in _lib.lib.lbswim_last_error()
    # few spread bins, but an axis beyond the gather's launch limits
    rc = _lib.lib.lbswim_spread_forces_noalloc(
        C.c_void_p(r.data_ptr()), C.c_void_p(r.data_ptr()), 1, 1e-3, 0.5, 4, 1000000, 4,
        C.c_void_p(force.data_ptr()), 0, None)
    assert rc == -1 and b"limit" in _lib.lib.lbswim_last_error()
    torch.cuda.synchronize()
    assert float(force.abs().max()) == 0.0
