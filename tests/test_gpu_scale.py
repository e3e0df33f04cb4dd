"""Parity at the benchmark's own sizes.

The small fixtures elsewhere never reach the code paths that switch on size:
the 64-bit slab counts, the slab buckets at real end densities, tracer
re-binning over 1M tracers, the carried force sums.  Here:

* 256^3 with 65,536 swimmers and 1,048,576 tracers (the benchmark workload,
  bench.workload): the FP64 exact mode equals the oracle bit for bit after 3
  coupled steps; the default FP64 path holds the FP64 parity tolerances; FP32
  storage tracks the FP64 path over 20 steps within the FP32 bounds below.
* 384^3 with 262,144 swimmers in 16 arrays of their own P and alpha and
  1,048,576 tracers (the precision-study problem, precision_study.problem):
  FP32, BF16 and FP16 storage against the FP64 path after 100 steps, within
  the per-field bounds below.
"""
import os

import numpy as np
import pytest

import bench
import oracle as O
import precision_study as PS
from gpu_harness import build_gpu, snapshot
from helpers import rel_l2, rel_max
from test_gpu_parity import EXACT, compare

pytestmark = pytest.mark.gpu

C1 = (256, 256, 256)
ORACLE_STEPS = 3
F32_STEPS = 20
C2_STEPS = 100
KEYS = ("rho", "u", "force", "f", "sw_r", "sw_v", "sw_n", "tr_r", "tr_v")

# FP32 against FP64 at 256^3 after 20 steps: rho, f relative L2; u, force
# max-norm error over the field's max; positions (periodic, sites) and
# velocities (lattice units) max abs error
F32_BOUNDS = {"rho": 1e-6, "f": 1e-6, "u": 1e-4, "force": 1e-6, "pos": 1e-5, "vel": 1e-6,
              "n": 1e-4}
# 384^3 after 100 steps, storage format -> (rho rel L2, u rel L2, max swimmer
# position error, max tracer position error)
C2_BOUNDS = {"f32": (1e-9, 1e-5, 1e-4, 1e-5),
             "bf16": (1e-6, 5e-3, 1e-4, 1e-4),
             "f16": (1e-6, 2e-3, 1e-4, 1e-4)}


def _periodic_err(a, b, size):
    box = np.asarray(size, dtype=float).reshape(3, 1)
    d = (a - b + box / 2) % box - box / 2
    return float(np.abs(d).max())


@pytest.fixture(scope="module")
def c1_case():
    nsw, ntr = bench.scaled_counts(256)
    return bench.workload(C1, nsw, ntr)


@pytest.fixture(scope="module")
def c1_oracle(c1_case):
    O.set_threads(os.cpu_count())
    orc = O.make_system(c1_case)
    orc.step(ORACLE_STEPS)
    snap = orc.snapshot()
    del orc
    return snap


def test_c1_f64_exact_mode_equals_oracle_bit_for_bit(c1_case, c1_oracle):
    lat, sw, tr, system = build_gpu(c1_case, "f64", compat=EXACT)
    system.Step(ORACLE_STEPS)
    g = snapshot(lat, sw, tr)
    for k in KEYS:
        assert np.array_equal(g[k], c1_oracle[k]), k


def test_c1_f64_default_path_within_parity_tolerance(c1_case, c1_oracle):
    lat, sw, tr, system = build_gpu(c1_case, "f64")
    system.Step(ORACLE_STEPS)
    compare(snapshot(lat, sw, tr), c1_oracle)


def test_c1_f32_tracks_f64(c1_case):
    ref = build_gpu(c1_case, "f64")
    got = build_gpu(c1_case, "f32")
    ref[3].Step(F32_STEPS)
    got[3].Step(F32_STEPS)
    r, g = snapshot(*ref[:3]), snapshot(*got[:3])
    B = F32_BOUNDS
    assert rel_l2(g["rho"], r["rho"]) <= B["rho"]
    assert rel_l2(g["f"], r["f"]) <= B["f"]
    assert rel_max(g["u"], r["u"]) <= B["u"]
    assert rel_l2(g["force"], r["force"]) <= B["force"] and np.abs(r["force"]).max() > 0
    assert _periodic_err(g["sw_r"], r["sw_r"], C1) <= B["pos"]
    assert _periodic_err(g["tr_r"], r["tr_r"], C1) <= B["pos"]
    assert np.abs(g["sw_v"] - r["sw_v"]).max() <= B["vel"]
    assert np.abs(g["tr_v"] - r["tr_v"]).max() <= B["vel"]
    assert np.abs(g["sw_n"] - r["sw_n"]).max() <= B["n"]


@pytest.fixture(scope="module")
def c2_problem():
    return PS.problem(384, 262144, 1048576, 16)


@pytest.fixture(scope="module")
def c2_f64(c2_problem):
    return PS.run(c2_problem, "f64", C2_STEPS)


@pytest.mark.parametrize("precision", ["f32", "bf16", "f16"])
def test_c2_reduced_precision_against_f64(c2_problem, c2_f64, precision):
    got = PS.run(c2_problem, precision, C2_STEPS)
    e = PS.compare(c2_f64, got, 384.0)
    rho_b, u_b, sw_b, tr_b = C2_BOUNDS[precision]
    print(precision, e)
    assert e["rho_rel_l2"] <= rho_b
    assert e["u_rel_l2"] <= u_b
    assert e["swimmer_pos_max_err"] <= sw_b
    assert e["tracer_pos_max_err"] <= tr_b
    # mass is conserved by the FP64 sums of every format
    m0 = float(c2_problem["rho"].sum())
    assert abs(got["mass_momentum"][0] - m0) <= {"f32": 1e-9, "bf16": 1e-6, "f16": 1e-6}[
        precision] * m0
