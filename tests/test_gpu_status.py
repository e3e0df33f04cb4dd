"""Failure detection without a GPU fault: the sticky status word and the
validation of uploads.

A non-finite density is uploaded (plain arithmetic on a finite-size field, no
bad index anywhere): the step and CalcHydro kernels flag it, the status stays
set until read with clear, and a healthy lattice reports nothing.  Particle
uploads with a NaN or an infinity are rejected (checked on the device, on a
staged copy) and leave the field as it was.
"""
import numpy as np
import pytest

import oracle as O
from gpu_harness import build_gpu
from lbswim import _lib, swimmers, tracers

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["f64", "f32", "bf16"])
def test_nonfinite_density_sets_the_sticky_status(precision):
    case = O.random_case((8, 12, 32), 4, 30, seed=4)
    lat, sw, tr, system = build_gpu(case, precision)
    system.Step(2)
    assert lat.status() == 0
    N = lat.addr.n
    rho = np.broadcast_to(case["rho"], (N,)).copy()
    rho[N // 3] = np.nan
    lat.rho[:] = rho.reshape(lat.rho.shape)
    lat.rho.H2D()
    lat.InitFromHydro()
    system.Step(1)
    st = lat.status(clear=True)
    assert st & _lib.STATUS_NONFINITE
    assert lat.status() == 0  # cleared
    # a fresh lattice of the same case stays clean
    lat2, _, _, system2 = build_gpu(case, precision)
    system2.Step(3)
    assert lat2.status() == 0


def test_nonfinite_particle_uploads_are_rejected():
    cp = swimmers.CommonParams()
    sw = swimmers.Array(5, cp)
    sw.r[:] = 1.0
    sw.H2D()
    before = sw.r.data.copy()
    sw.r[1, 2] = np.inf
    with pytest.raises(_lib.LbswimError, match="non-finite"):
        sw.r.H2D()
    sw.n[:] = 0.0
    sw.n[2, 0] = np.nan
    with pytest.raises(_lib.LbswimError, match="non-finite"):
        sw.n.H2D()
    sw.r.D2H()
    assert np.array_equal(sw.r.data, before)  # nothing was copied
    tr = tracers.Array(7)
    tr.r[:] = 2.0
    tr.r.H2D()
    tr.r[0, 3] = np.nan
    with pytest.raises(_lib.LbswimError, match="non-finite"):
        tr.r.H2D()
    tr.r.D2H()
    assert np.all(tr.r.data == 2.0)  # nothing was copied
    tr.v[:] = np.nan  # velocities are outputs of the move; not checked
    tr.v.H2D()
