"""The CPU oracle, pinned against the reference's own kernels.

The golden fixtures in tests/golden/ were produced by the reference's CUDA
sources built for the host (oracle/build_ref.py, tests/golden/make_golden.py).
The oracle restatement must reproduce them bit for bit on x86-64 (same
compiler, -ffp-contract=off); elsewhere it must agree to 1e-13.
"""
import hashlib
import platform

import numpy as np
import pytest

import oracle as O
from helpers import GOLDEN_CASES, golden_case, load_golden

EXACT = platform.machine() in ("x86_64", "AMD64")


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype=np.float64).tobytes()).hexdigest()


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_oracle_matches_reference_fixture(name):
    g = load_golden(name)
    case = golden_case(name)
    sysm = O.make_system(case)
    done = 0
    for t in g["snaps"]:
        sysm.step(int(t) - done)
        done = int(t)
        s = sysm.snapshot()
        for key in ("rho", "u", "force", "f", "sw_r", "sw_v", "sw_n", "tr_r", "tr_v"):
            if key not in s:
                continue
            ref_digest = str(g["%s@%d#sha" % (key, t)])
            if key in ("rho", "u", "force", "f"):
                sel = s[key][..., g["sites"]]
            elif key.startswith("tr_"):
                sel = s[key][:, g["tracers"]]
            else:
                sel = s[key]
            ref_vals = g["%s@%d" % (key, t)]
            if EXACT:
                assert np.array_equal(sel, ref_vals), (name, key, t)
                assert sha(s[key]) == ref_digest, (name, key, t)
            else:
                np.testing.assert_allclose(sel, ref_vals, rtol=1e-13, atol=1e-15)


def test_philox_known_answers():
    # Random123 known-answer vectors for philox4x32-10.
    assert O.philox4x32([0, 0, 0, 0], [0, 0]) == [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]
    assert O.philox4x32([0xffffffff] * 4, [0xffffffff] * 2) == [
        0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]
    assert O.philox4x32([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344],
                        [0xa4093822, 0x299f31d0]) == [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1]


def test_rng_stream_statistics():
    u = np.array([O.rng_uniform(99, i, t) for i in range(200) for t in range(50)])
    assert u.min() > 0 and u.max() <= 1
    assert abs(u.mean() - 0.5) < 0.01
    assert abs(np.mean(u < 0.05) - 0.05) < 0.01
    g = np.array([O.rng_normal3(7, i, t) for i in range(300) for t in range(20)])
    assert abs(g.mean()) < 0.03 and abs(g.std() - 1) < 0.03
    # tumble directions are isotropic
    n = g / np.linalg.norm(g, axis=1, keepdims=True)
    assert np.all(np.abs(n.mean(axis=0)) < 0.04)


def test_peskin_known_answers():
    g = load_golden("peskin")
    phi = np.array([O.peskin_delta(x) for x in g["x"]])
    if EXACT:
        assert np.array_equal(phi, g["phi"])
    else:
        np.testing.assert_allclose(phi, g["phi"], rtol=1e-15, atol=1e-17)


@pytest.mark.parametrize("r", [0.0, 0.25, 0.5, 0.731, 1.0 - 1e-9, 3.999])
def test_peskin_stencil_moments(r):
    x0 = np.ceil(r - 2.0)
    xs = x0 + np.arange(4)
    phi = np.array([O.peskin_delta(r - x) for x in xs])
    assert abs(phi.sum() - 1.0) < 1e-14          # partition of unity
    assert abs(((xs - r) * phi).sum()) < 1e-14  # first moment vanishes
    assert abs((phi[0::2].sum()) - 0.5) < 1e-14  # even/odd condition of the 4-point delta


def test_d3q15_tables():
    P = O.params_dict(O.params(0.8, 0.8))
    mm, mmi = P["mm"], P["mmi"]
    np.testing.assert_allclose(mm @ mmi, np.eye(15), atol=1e-14)
    np.testing.assert_allclose(mmi[:, 0], P["w"], atol=0)
    assert P["w"].sum() == pytest.approx(1.0, abs=1e-15)
    ci = P["ci"]
    for p in range(15):
        assert np.array_equal(ci[P["complement"][p]], -ci[p])
    np.testing.assert_allclose((P["w"][:, None] * ci * ci).sum(0), P["cs2"], atol=1e-15)


def test_oracle_conserves_mass_and_balances_momentum():
    case = O.random_case((12, 10, 14), 30, 0, seed=3, u_amp=0.01)
    s = O.make_system(case)
    m0 = s.f.reshape(15, -1).sum()
    s.step(20)
    m1 = s.f.reshape(15, -1).sum()
    assert abs(m1 - m0) / m0 < 1e-13
    # every dipole exerts zero net force on the fluid
    assert np.abs(s.force.reshape(3, -1).sum(axis=1)).max() < 1e-15


def test_zero_velocity_tracers_stay_put():
    case = O.random_case((8, 8, 8), 0, 100, seed=9)
    case["rho"] = 1.0
    s = O.make_system(case)
    r0 = s.tr["r"].copy()
    s.step(10)
    # rest equilibrium is a fixed point up to rounding
    assert np.abs(s.tr["r"] - r0).max() < 1e-12
