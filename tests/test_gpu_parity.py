"""FP64 parity of the CUDA path with the oracle and the reference's fixtures.

With LBSWIM_COMPAT_EXACT_F64 every FP64 array is the oracle's, bit for bit,
and hashes to the digest that the reference's own host build wrote into the
fixture.  The default FP64 path (butterfly moment transform and fused
multiply-adds in the lattice kernels; one square root per axis for the Peskin
weights and fused multiply-adds in the particle moves) is held to:
  rho, f        relative L2 <= 1e-12;
  u, force, v   relative L2 normalised by the field's max magnitude <= 1e-10
                (u is a small difference of O(0.1) sums, 1e-8..1e-5 here, so
                a one-ulp change of a distribution moves it by 1e-12..1e-11 of
                max|u|);
                max-norm error relative to the max magnitude <= 1e-10;
  r, n          per coordinate, relative to max(1, |x|), <= 1e-12.
Tumble decisions and cell indices are compared exactly.
"""
import hashlib

import numpy as np
import pytest

import oracle as O
from lbswim import _lib
from gpu_harness import build_gpu, snapshot
from helpers import (GOLDEN_CASES, TOL_F64, golden_case, load_golden, rel_l2, rel_l2_maxnorm,
                     rel_max)

pytestmark = pytest.mark.gpu
TOL_MAXNORM = 1e-10
TOL_SMALL_FIELD = 1e-10  # u, force, v of the default FP64 path


def particle_err(a, b):
    return float(np.max(np.abs(a - b) / np.maximum(1.0, np.abs(b)))) if a.size else 0.0


def compare(gs, os_, tol=TOL_F64):
    errs = {"rho": rel_l2(gs["rho"], os_["rho"]), "f": rel_l2(gs["f"], os_["f"]),
            "u": rel_l2_maxnorm(gs["u"], os_["u"]),
            "force": rel_l2_maxnorm(gs["force"], os_["force"])}
    for k in ("sw_r", "sw_v", "sw_n", "tr_r", "tr_v"):
        if k in os_:
            if k.endswith("_v"):
                errs[k] = rel_l2_maxnorm(gs[k], os_[k])
            else:
                errs[k] = particle_err(gs[k], os_[k])
    small = ("u", "force", "sw_v", "tr_v")
    bad = {k: v for k, v in errs.items() if not v <= (TOL_SMALL_FIELD if k in small else tol)}
    assert not bad, bad
    for k in ("u", "force"):
        assert rel_max(gs[k], os_[k]) <= TOL_MAXNORM, k
    return errs


EXACT = _lib.COMPAT_INIT_SXZ | _lib.COMPAT_EXACT_F64


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype=np.float64).tobytes()).hexdigest()


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_f64_exact_mode_is_the_reference_bit_for_bit(name):
    g = load_golden(name)
    case = golden_case(name)
    lat, sw, tr, system = build_gpu(case, "f64", compat=EXACT)
    orc = O.make_system(case)
    done = 0
    for t in g["snaps"]:
        t = int(t)
        system.Step(t - done)
        orc.step(t - done)
        done = t
        gs, os_ = snapshot(lat, sw, tr), orc.snapshot()
        for key in ("rho", "u", "force", "f", "sw_r", "sw_v", "sw_n", "tr_r", "tr_v"):
            if key not in os_:
                continue
            assert np.array_equal(gs[key], os_[key]), (name, key, t)
            assert sha(gs[key]) == str(g["%s@%d#sha" % (key, t)]), (name, key, t)


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_f64_matches_oracle_and_reference_fixture(name):
    g = load_golden(name)
    case = golden_case(name)
    lat, sw, tr, system = build_gpu(case)
    orc = O.make_system(case)
    done = 0
    for t in g["snaps"]:
        t = int(t)
        system.Step(t - done)
        orc.step(t - done)
        done = t
        assert lat.time_step == t
        gs = snapshot(lat, sw, tr)
        compare(gs, orc.snapshot())
        # against the reference's own values at the fixture's sample points
        sites, tsel = g["sites"], g["tracers"]
        assert rel_l2(gs["rho"][sites], g["rho@%d" % t]) <= TOL_F64
        assert rel_l2(gs["f"][:, sites], g["f@%d" % t]) <= TOL_F64
        assert rel_l2_maxnorm(gs["u"][:, sites], g["u@%d" % t]) <= TOL_SMALL_FIELD
        if sw is not None:
            assert particle_err(gs["sw_r"], g["sw_r@%d" % t]) <= TOL_F64
            assert particle_err(gs["sw_n"], g["sw_n@%d" % t]) <= TOL_F64
        if tr is not None:
            assert particle_err(gs["tr_r"][:, tsel], g["tr_r@%d" % t]) <= TOL_F64


def test_single_ops_equal_fused_system_step():
    case = golden_case("rand_small")
    a = build_gpu(case)
    b = build_gpu(case)
    lat, sw, tr, _ = a
    for _ in range(12):
        lat.ZeroForce()
        sw.AddForces(lat)
        tr.AddForces(lat)
        lat.Step()
        lat.CalcHydro()
        sw.Move(lat)
        tr.Move(lat)
    b[3].Step(12)
    sa, sb = snapshot(*a[:3]), snapshot(*b[:3])
    for k in sa:
        assert np.array_equal(sa[k], sb[k]), k


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_bitwise_deterministic(precision):
    case = O.random_case((24, 20, 36), 300, 500, seed=77, alpha=0.2)
    runs = []
    for _ in range(2):
        lat, sw, tr, system = build_gpu(case, precision)
        system.Step(25)
        runs.append(snapshot(lat, sw, tr))
    for k in runs[0]:
        assert np.array_equal(runs[0][k], runs[1][k]), k


def test_tumble_decisions_bit_exact():
    # With rotational advection off an orientation changes only when it tumbles.
    case = O.random_case((16, 16, 16), 2000, 0, seed=5, alpha=0.3, rot_off=True)
    lat, sw, tr, system = build_gpu(case)
    orc = O.make_system(case)
    for step in range(4):
        sw.D2H()
        n_before = sw.n.data.copy()
        o_before = orc.sw["nvec"].reshape(3, -1).copy()
        system.Step(1)
        orc.step(1)
        sw.D2H()
        g_t = np.any(sw.n.data != n_before, axis=0)
        o_t = np.any(orc.sw["nvec"].reshape(3, -1) != o_before, axis=0)
        assert np.array_equal(g_t, o_t), step
        assert 0.2 < g_t.mean() < 0.4
        assert particle_err(sw.n.data, orc.sw["nvec"].reshape(3, -1)) <= TOL_F64


@pytest.mark.parametrize("name", ["c0_readme", "c1_density_32"])
def test_cell_indices_bit_exact(name):
    case = golden_case(name)
    lat, sw, tr, system = build_gpu(case)
    orc = O.make_system(case)
    system.Step(40)
    orc.step(40)
    gs, os_ = snapshot(lat, sw, tr), orc.snapshot()
    for key in ("sw_r", "tr_r"):
        g, o = gs[key], os_[key]
        # stencil origins as the reference computes them (interp.cu:24)
        cg, co = np.ceil(g - 2.0), np.ceil(o - 2.0)
        # positions within 1e-12 of a cell boundary are only defined to the FP64 tolerance
        ambiguous = np.abs(o - np.round(o)) < 1e-12
        assert np.array_equal(cg[~ambiguous], co[~ambiguous]), key
        assert np.count_nonzero(~ambiguous) > 0


def test_mass_conserved_f64():
    case = O.random_case((20, 24, 28), 64, 0, seed=12, u_amp=0.01)
    lat, sw, tr, system = build_gpu(case)
    lat.fOld.D2H()
    m0 = lat.fOld.data.sum()
    system.Step(50)
    lat.fOld.D2H()
    assert abs(lat.fOld.data.sum() - m0) / m0 < 1e-12
    lat.force.D2H()
    assert np.abs(lat.force.data.reshape(3, -1).sum(axis=1)).max() < 1e-15


def test_init_from_hydro_sxz_compat_switch():
    case = O.random_case((6, 7, 8), 0, 0, seed=4, u_amp=0.05)
    lat, _, _, _ = build_gpu(case)
    lat.fOld.D2H()
    ref = O.make_system(case, compat_sxz=True).f.reshape(15, -1)
    assert rel_l2(lat.fOld.data.reshape(15, -1), ref) <= TOL_F64
    lat2, _, _, _ = build_gpu(case, compat=0)
    lat2.fOld.D2H()
    fixed = O.make_system(case, compat_sxz=False).f.reshape(15, -1)
    assert rel_l2(lat2.fOld.data.reshape(15, -1), fixed) <= TOL_F64
    assert rel_l2(ref, fixed) > 1e-6


def test_rng_draws_bit_exact():
    from lbswim import _lib
    for seed, step in ((23774, 0), (1234, 7), (2 ** 40 + 5, 2 ** 33 + 1)):
        u, g = _lib.rng_draws(seed, 257, step)
        ou = np.array([O.rng_uniform(seed, i, step) for i in range(257)], dtype=np.float32)
        og = np.array([O.rng_normal3(seed, i, step) for i in range(257)]).T
        assert np.array_equal(u, ou), (seed, step)
        assert np.max(np.abs(g - og)) <= 1e-14


@pytest.mark.parametrize("shape", [(16, 12, 20), (5, 7, 3), (3, 2, 9)])
def test_interp_velocity_matches_oracle(shape):
    case = O.random_case(shape, 0, 0, seed=4, u_amp=0.02)
    lat, _, _, _ = build_gpu(case)
    lat.Step()
    lat.CalcHydro()
    lat.u.D2H()
    u = np.ascontiguousarray(lat.u.data.reshape(-1))
    rng = np.random.default_rng(1)
    L = np.array(shape, dtype=float).reshape(3, 1)
    pts = np.concatenate([rng.random((3, 200)) * L, np.floor(rng.random((3, 20)) * L),
                          L - 1e-9 + 0 * rng.random((3, 5)), -0.3 + 0 * rng.random((3, 3))], axis=1)
    v = lat.interp_velocity(pts)
    ov = np.zeros_like(v)
    for i in range(pts.shape[1]):
        out = np.zeros(3)
        O.lib().orc_interp_velocity(O._I3(*shape), O._p(u), O._p(np.ascontiguousarray(pts[:, i])),
                                    O._p(out))
        ov[:, i] = out
    assert rel_l2_maxnorm(v, ov) <= TOL_F64 and rel_max(v, ov) <= TOL_MAXNORM
