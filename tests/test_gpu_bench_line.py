"""bench.py on the GPU: one small run prints the one JSON line of the benchmark
contract, with every key the contract asks for and self-consistent figures
(the device-timed value from its own step time, the roofline fraction from
its achieved and peak bandwidth, the end-to-end figure below the device one).
"""
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_bench_prints_the_contract_line():
    side, steps = 64, 4
    r = subprocess.run(
        [sys.executable, os.path.join(ROOT, "bench.py"), "--size", str(side), "--steps",
         str(steps), "--warmup", "3", "--cpu-seconds", "0.5", "--f64-steps", "2",
         "--ens-members", "6", "--ens-steps", "20", "--ens-check", "2", "--ens-f64-steps", "2",
         "--serve-seconds", "1", "--serve-rate", "20", "--serve-rate-low", "0"],
        capture_output=True, text=True, timeout=900, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-3000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.strip().startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
              "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config", "clocks",
              "e2e", "gpu_launches", "roofline", "step_roofline", "cpu_baseline", "f64",
              "ensemble", "serving"):
        assert k in d, k
    assert d["unit"] == "GLUPS" and d["higher_is_better"] is True and d["scaling"] == "weak"
    assert d["steps"] == steps and d["warmup"] == 3 and d["n_gpus"] == 1
    assert d["dtype"] == "f32" and d["config"]["lattice"] == [side] * 3
    # value: sites x steps over the timed steps
    assert abs(d["value"] - side ** 3 / (d["ms_per_step"] / 1e3) / 1e9) <= 1e-6 * d["value"]
    roof = d["roofline"]
    assert roof["bound"] == "hbm" and roof["unit"] == "GB/s" and roof["peak"] > 0
    assert abs(roof["frac"] - roof["achieved"] / roof["peak"]) <= 1e-9
    assert 0 < roof["frac"] < 1.5 and roof["kernel"] == "k_fused_step"
    assert roof["timed_launches"].startswith("1 of %d" % steps)  # every 4th of 4 steps
    e2e = d["e2e"]
    assert e2e["unit"] == "GLUPS" and 0 < e2e["value"] < d["value"]
    assert e2e["h2d_bytes_per_step"] > 0 and e2e["d2h_bytes_per_step"] > 0
    # the library's own kernels ran in the timed region: at least the step
    # kernel, the swimmer move and the tracer move per step
    assert d["gpu_launches"] >= 3 * steps
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["value"] > 0 and cb["cores"] >= 1
    assert d["f64"]["precision"] == "f64" and d["f64"]["glups"] > 0
    assert d["ensemble"]["members"] == 6 and d["ensemble"]["batched_glups"] > 0
    assert d["ensemble"]["u_rel_l2_vs_f64"] < 1e-5
    assert d["serving"]["batched_f32"]["arrivals"] >= 0
    assert "sm_mhz" in d["clocks"] and "reasons" in d["clocks"]
