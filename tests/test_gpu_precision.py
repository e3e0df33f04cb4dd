"""Reduced-precision storage against the FP64 oracle, with the stated bounds.

FP32 stores f - w_i rho0; BF16 and FP16 store (f - w_i rho0) / w_i; all three
collide in FP32.  Positions stay FP64.
"""
import numpy as np
import pytest

import oracle as O
from gpu_harness import build_gpu, snapshot
from helpers import rel_l2, rel_max

pytestmark = pytest.mark.gpu

# (precision, max rel-L2 of rho, max |u - u_ref| / max|u_ref|) after 200 steps
BOUNDS = [("f32", 1e-6, 1e-5), ("f16", 1e-4, 3e-2), ("bf16", 1e-3, 3e-1)]


@pytest.mark.parametrize("precision,rho_tol,u_tol", BOUNDS)
def test_reduced_precision_error_bounds(precision, rho_tol, u_tol):
    case = O.random_case((24, 24, 24), 60, 400, seed=8, alpha=0.01)
    lat, sw, tr, system = build_gpu(case, precision)
    orc = O.make_system(case)
    system.Step(200)
    orc.step(200)
    gs, os_ = snapshot(lat, sw, tr), orc.snapshot()
    e_rho = rel_l2(gs["rho"], os_["rho"])
    e_u = rel_max(gs["u"], os_["u"])
    print(precision, "rho", e_rho, "u", e_u)
    assert e_rho <= rho_tol and e_u <= u_tol


def test_f32_mass_conservation():
    case = O.random_case((32, 16, 48), 100, 0, seed=2, u_amp=0.01)
    lat, sw, tr, system = build_gpu(case, "f32")
    lat.fOld.D2H()
    m0 = lat.fOld.data.sum()
    system.Step(100)
    lat.fOld.D2H()
    assert abs(lat.fOld.data.sum() - m0) / m0 < 1e-7


@pytest.mark.parametrize("shape", [(5, 7, 3), (17, 9, 33), (40, 3, 16), (1, 8, 8)])
def test_f32_ragged_shapes_match_oracle(shape):
    case = O.random_case(shape, 5, 20, seed=sum(shape), u_amp=0.01)
    lat, sw, tr, system = build_gpu(case, "f32")
    orc = O.make_system(case)
    system.Step(20)
    orc.step(20)
    gs, os_ = snapshot(lat, sw, tr), orc.snapshot()
    assert rel_l2(gs["rho"], os_["rho"]) < 1e-6
    assert rel_max(gs["u"], os_["u"]) < 1e-4
    assert rel_l2(gs["f"], os_["f"]) < 1e-6
