"""Host <-> device copies of the lattice fields through the C ABI.

A page-locked host buffer is read or written by the conversion kernels
themselves (the buffer is mapped into the device's address space); a pageable
one goes through the staging buffer in chunks.  Both must give the same bits,
for every field and storage format, and the FP32 fields must hold the FP64
values rounded once (rho as rho - rho0).
"""
import numpy as np
import pytest

from lbswim import _lib, lb

pytestmark = pytest.mark.gpu

SHAPE = (19, 23, 37)  # N = 16,169: not a multiple of the 32-site blocks
COMPONENTS = {_lib.FIELD_RHO: 1, _lib.FIELD_U: 3, _lib.FIELD_FORCE: 3,
              _lib.FIELD_FOLD: 15, _lib.FIELD_FNEW: 15}


def _h2d(lat, field, buf):
    _lib.check(_lib.lib.lbswim_lattice_h2d(lat._h, field, _lib.dptr(buf)))


def _d2h(lat, field, buf):
    _lib.check(_lib.lib.lbswim_lattice_d2h(lat._h, field, _lib.dptr(buf)))


def _values(field, n, rng):
    if field == _lib.FIELD_RHO:
        return 1.0 + 1e-3 * rng.standard_normal(n)
    if field in (_lib.FIELD_FOLD, _lib.FIELD_FNEW):
        w = np.array([2 / 9] + [1 / 9] * 6 + [1 / 72] * 8)
        return (w[:, None] * (1.0 + 1e-3 * rng.standard_normal((15, n // 15)))).reshape(-1)
    return 1e-3 * rng.standard_normal(n)


@pytest.mark.parametrize("precision", ["f32", "bf16", "f16"])
@pytest.mark.parametrize("field", sorted(COMPONENTS))
def test_pinned_and_pageable_buffers_give_the_same_bits(precision, field):
    lat = lb.Lattice(*SHAPE, 0.8, 0.8, precision=precision)
    N = int(np.prod(SHAPE))
    n = COMPONENTS[field] * N
    vals = _values(field, n, np.random.default_rng(field))
    pageable = np.ascontiguousarray(vals)
    pinned = _lib.pinned_zeros(n)
    pinned[:] = vals

    out = {}
    for src_name, src in (("pageable", pageable), ("pinned", pinned)):
        _h2d(lat, field, src)
        for dst_name in ("pageable", "pinned"):
            dst = np.zeros(n) if dst_name == "pageable" else _lib.pinned_zeros(n)
            _d2h(lat, field, dst)
            out[src_name, dst_name] = np.array(dst)
    ref = out["pageable", "pageable"]
    for k, v in out.items():
        assert np.array_equal(v, ref), k

    if precision == "f32" and field in (_lib.FIELD_RHO, _lib.FIELD_U, _lib.FIELD_FORCE):
        if field == _lib.FIELD_RHO:
            rho0 = lat.rho0
            want = (vals - rho0).astype(np.float32).astype(np.float64) + rho0
        else:
            want = vals.astype(np.float32).astype(np.float64)
        assert np.array_equal(ref, want)
    else:
        # one rounding to the storage format (BF16 / FP16 hold the deviation
        # from w_i rho0 over w_i)
        tol = {"f32": 1e-7, "bf16": 1e-2, "f16": 1e-3}[precision]
        scale = np.abs(vals).max()
        assert np.abs(ref - vals).max() <= tol * scale


def test_rho_and_u_uploads_leave_each_other_alone():
    # rho and u share the packed float4 of a site: an upload of one keeps the
    # other's bits
    lat = lb.Lattice(*SHAPE, 0.8, 0.8, precision="f32")
    N = int(np.prod(SHAPE))
    rng = np.random.default_rng(5)
    rho = _lib.pinned_zeros(N)
    rho[:] = 1.0 + 1e-3 * rng.standard_normal(N)
    u = _lib.pinned_zeros(3 * N)
    u[:] = 1e-3 * rng.standard_normal(3 * N)
    _h2d(lat, _lib.FIELD_RHO, rho)
    _h2d(lat, _lib.FIELD_U, u)
    got_rho, got_u = np.zeros(N), np.zeros(3 * N)
    _d2h(lat, _lib.FIELD_RHO, got_rho)
    _d2h(lat, _lib.FIELD_U, got_u)
    rho0 = lat.rho0
    assert np.array_equal(got_rho, (rho - rho0).astype(np.float32).astype(np.float64) + rho0)
    assert np.array_equal(got_u, u.astype(np.float32).astype(np.float64))
    u2 = np.ascontiguousarray(-u)  # pageable this time
    _h2d(lat, _lib.FIELD_U, u2)
    _d2h(lat, _lib.FIELD_RHO, got_rho)
    assert np.array_equal(got_rho, (rho - rho0).astype(np.float32).astype(np.float64) + rho0)
