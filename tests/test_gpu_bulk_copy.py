"""The step kernel's bulk-copied rows (cp.async.bulk into shared memory, with
LBSWIM_COMPAT_BULK_COPY when nz is a multiple of 32) give the same bits as its
per-thread loads.

Same workload twice, one lattice with the flag: after system steps with
pending forces, steps from a materialised dense force, and ragged slabs in x
and y, every field and particle array is equal bit for bit.
"""
import numpy as np
import pytest

import oracle as O
from gpu_harness import build_gpu, snapshot
from lbswim import _lib

pytestmark = pytest.mark.gpu


def _pair(case, precision):
    a = build_gpu(case, precision, compat=_lib.COMPAT_INIT_SXZ | _lib.COMPAT_BULK_COPY)
    b = build_gpu(case, precision)
    return a, b


@pytest.mark.parametrize("precision", ["f32", "bf16", "f16"])
@pytest.mark.parametrize("shape", [(40, 24, 64), (37, 13, 32), (5, 9, 96)])
def test_bulk_copied_rows_equal_per_thread_loads(precision, shape):
    case = O.random_case(shape, 150, 400, seed=sum(shape), alpha=0.1, u_amp=0.01, P=2e-3,
                         l=0.4)
    a, b = _pair(case, precision)
    for lat, sw, tr, system in (a, b):
        system.Step(4)
        # a step from a dense force: read it back (materialises it), add to it
        lat.ZeroForce()
        sw.AddForces(lat)
        lat.force.D2H()
        lat.Step()
        lat.CalcHydro()
        sw.Move(lat)
        tr.Move(lat)
        system.Step(3)
    sa, sb = snapshot(*a[:3]), snapshot(*b[:3])
    for k in sa:
        assert np.array_equal(sa[k], sb[k]), k
    assert a[0].status() == 0 and b[0].status() == 0
