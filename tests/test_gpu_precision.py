"""Reduced-precision storage against the FP64 oracle, with the stated bounds.

FP32 stores f - w_i rho0; BF16 and FP16 store (f - w_i rho0) / w_i; all three
collide in FP32.  Particle positions are stored in FP64 and advanced in Q44
fixed point; velocities are interpolated in FP32.
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


@pytest.mark.parametrize("precision", ["f32", "bf16"])
def test_wide_site_offsets_give_the_same_bits(precision):
    # Lattices of 15 N >= 2^31 sites (N >= 2^31 for the moves) take the
    # 64-bit-offset instances of the step and move kernels; the compat flag
    # makes a small lattice take them too, and nothing but the offsets' type
    # may change: every field ends the same, bit for bit
    from lbswim import _lib
    case = O.random_case((24, 20, 36), 300, 700, seed=12, alpha=0.1, u_amp=0.01)
    narrow = build_gpu(case, precision)
    wide = build_gpu(case, precision, compat=_lib.COMPAT_INIT_SXZ | _lib.COMPAT_WIDE_INDEX)
    for lat, sw, tr, system in (narrow, wide):
        system.Step(70)  # crosses a tracer re-binning
        lat.ZeroForce()
        sw.AddForces(lat)
        lat.force.D2H()
    a, b = snapshot(*narrow[:3]), snapshot(*wide[:3])
    for k in a:
        assert np.array_equal(a[k], b[k]), k
    assert np.abs(a["force"]).max() > 0


@pytest.mark.parametrize("shape", [(5, 7, 3), (17, 9, 33), (40, 3, 16), (1, 8, 8), (9, 7, 5), (33, 10, 40)])
def test_f32_ragged_shapes_match_oracle(shape):
    case = O.random_case(shape, 60, 20, seed=sum(shape), u_amp=0.01)
    lat, sw, tr, system = build_gpu(case, "f32")
    orc = O.make_system(case)
    system.Step(20)
    orc.step(20)
    gs, os_ = snapshot(lat, sw, tr), orc.snapshot()
    assert rel_l2(gs["rho"], os_["rho"]) < 1e-6
    assert rel_max(gs["u"], os_["u"]) < 1e-4
    assert rel_l2(gs["f"], os_["f"]) < 1e-6


def _spread_case():
    return O.random_case((40, 24, 36), 400, 300, seed=21, alpha=0.1, P=2e-3, l=0.4)


@pytest.mark.parametrize("kind", ["sparse", "dense", "ragged", "folded"])
def test_f32_in_kernel_spread_equals_materialised_force(kind):
    # (a) the step kernel spreads the pending ends itself; (b) the force is read
    # back first, which writes the dense field, and the step then reads it.
    # The dense case puts more ends on one slab and one plane than the kernels'
    # shared-memory lists hold, which exercises their fallbacks; the ragged case
    # has partial slabs and tiles on every axis; the folded case also takes
    # the 64-bit sums with carries.
    case = {"sparse": _spread_case,
            "dense": lambda: O.random_case((16, 16, 16), 600, 50, seed=3, alpha=0.1, P=2e-3,
                                           l=0.4),
            "ragged": lambda: O.random_case((17, 9, 33), 120, 40, seed=9, alpha=0.1, P=2e-3,
                                            l=0.4),
            "folded": lambda: O.random_case((3, 8, 12), 2100, 10, seed=5, alpha=0.1, P=2e-3,
                                            l=0.4)}[kind]()
    a = build_gpu(case, "f32")
    b = build_gpu(case, "f32")
    for t in range(6):
        for lat, sw, tr, _ in (a, b):
            lat.ZeroForce()
            sw.AddForces(lat)
        b[0].force.D2H()
        for lat, sw, tr, _ in (a, b):
            lat.Step()
            lat.CalcHydro()
            sw.Move(lat)
            tr.Move(lat)
    sa, sb = snapshot(*a[:3]), snapshot(*b[:3])
    for k in sa:
        assert np.array_equal(sa[k], sb[k]), k


@pytest.mark.parametrize("folded", [False, True])
def test_f32_force_matches_f64_force(folded):
    # folded: an axis of 3 sites folds stencil nodes onto one site, and 4200
    # ends on every slab can put more than 65535 contributions on a site, so the
    # sums take their 64-bit form with carries
    case = (O.random_case((3, 8, 12), 2100, 10, seed=5, alpha=0.1, P=2e-3, l=0.4) if folded
            else _spread_case())
    l32 = build_gpu(case, "f32")
    l64 = build_gpu(case, "f64")
    for lat, sw, _, _ in (l32, l64):
        lat.ZeroForce()
        sw.AddForces(lat)
        lat.force.D2H()
    f32 = l32[0].force.data.reshape(3, -1)
    f64 = l64[0].force.data.reshape(3, -1)
    assert rel_l2(f32, f64) < 1e-6
    assert np.abs(f64).max() > 0


def test_f32_two_swimmer_arrays_accumulate():
    from lbswim import swimmers
    case = _spread_case()
    lat, sw, tr, system = build_gpu(case, "f32")
    s = case["swimmers"]
    cp = swimmers.CommonParams()
    for k in ("P", "l", "alpha", "mobility", "seed"):
        setattr(cp, k, s[k])
    sw2 = swimmers.Array(s["n"], cp)
    sw2.r[:] = s["r"]
    sw2.n[:] = s["nvec"]
    sw2.v[:] = 0
    sw2.H2D()
    lat.ZeroForce()
    sw.AddForces(lat)
    sw2.AddForces(lat)
    lat.force.D2H()
    both = lat.force.data.reshape(3, -1).copy()
    lat.ZeroForce()
    sw.AddForces(lat)
    lat.force.D2H()
    one = lat.force.data.reshape(3, -1).copy()
    assert rel_l2(both, 2 * one) < 1e-6
    # a step taken with two pending arrays equals one taken from the dense field
    system2 = build_gpu(case, "f32")
    lat.ZeroForce()
    sw.AddForces(lat)
    sw2.AddForces(lat)
    lat.Step()
    lat.CalcHydro()
    l2, s2a, _, _ = system2
    s2b = swimmers.Array(s["n"], cp)
    s2b.r[:] = s["r"]
    s2b.n[:] = s["nvec"]
    s2b.v[:] = 0
    s2b.H2D()
    l2.ZeroForce()
    s2a.AddForces(l2)
    s2b.AddForces(l2)
    l2.force.D2H()
    l2.Step()
    l2.CalcHydro()
    lat.u.D2H()
    l2.u.D2H()
    assert np.array_equal(lat.u.data, l2.u.data)


def _periodic_err(a, b, size):
    box = np.asarray(size, dtype=float).reshape(3, 1)
    d = (a - b + box / 2) % box - box / 2
    return np.abs(d).max()


@pytest.mark.parametrize("rot_off", [False, True])
def test_f32_particles_track_oracle(rot_off):
    """Swimmer and tracer states of the FP32 path (FP32 interpolation, Q44
    position updates, FP32 orientation updates and tumble directions) stay
    within FP32-level distance of the FP64 oracle; tumble decisions are the
    same draws."""
    shape = (32, 24, 40)
    case = O.random_case(shape, 300, 500, seed=31, alpha=0.2, u_amp=0.02, rot_off=rot_off)
    lat, sw, tr, system = build_gpu(case, "f32")
    orc = O.make_system(case)
    system.Step(20)
    orc.step(20)
    gs, os_ = snapshot(lat, sw, tr), orc.snapshot()
    assert _periodic_err(gs["sw_r"], os_["sw_r"], shape) < 1e-5
    assert _periodic_err(gs["tr_r"], os_["tr_r"], shape) < 1e-5
    assert np.abs(gs["tr_s"] - os_["tr_s"]).max() < 1e-5
    assert np.abs(gs["tr_v"] - os_["tr_v"]).max() < 1e-6
    assert np.abs(gs["sw_v"] - os_["sw_v"]).max() < 1e-6
    assert np.abs(gs["sw_n"] - os_["sw_n"]).max() < 1e-4
    assert np.allclose((gs["sw_n"] ** 2).sum(axis=0), 1.0, atol=1e-6)


@pytest.mark.parametrize("precision", ["f64", "f32", "bf16"])
def test_fp64_conservation_sums(precision):
    """Mass and momentum totals in FP64: equal to the sums of the read-back f,
    the same bits on every call, and conserved by the step (no force)."""
    case = O.random_case((24, 16, 20), 0, 0, seed=12, u_amp=0.01)
    lat, sw, tr, system = build_gpu(case, precision)
    c0 = lat.conservation()
    assert c0 == lat.conservation()
    lat.fOld.D2H()
    f = lat.fOld.data.reshape(15, -1)
    ci = np.array(lat.params.ci)
    assert abs(c0[0] - f.sum()) <= 1e-10 * abs(c0[0])
    for a in range(3):
        assert abs(c0[1 + a] - (ci[:, a:a + 1] * f).sum()) <= 1e-10 * abs(c0[0])
    for _ in range(10):
        lat.ZeroForce()
        lat.Step()
        lat.CalcHydro()
    c1 = lat.conservation()
    tol = {"f64": 1e-13, "f32": 1e-7, "bf16": 1e-3}[precision]
    assert abs(c1[0] - c0[0]) <= tol * abs(c0[0])
    for a in range(3):
        assert abs(c1[1 + a] - c0[1 + a]) <= tol * abs(c0[0])
