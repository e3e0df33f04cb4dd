"""bench.py --impl reference: the reference's method (the FP64 oracle, all host
threads) on a small cube, printed as one JSON line with the keys the
reference arm of the benchmark contract carries."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_json_line():
    r = subprocess.run(
        [sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--size", "24",
         "--steps", "2", "--warmup", "1"],
        capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.strip().startswith("{")]
    assert len(lines) == 1, r.stdout
    line = json.loads(lines[0])
    assert line["impl"] == "reference"
    assert line["unit"] == "GLUPS" and line["value"] > 0 and line["higher_is_better"] is True
    assert line["dtype"] == "f64" and line["config"]["precision"] == "f64"
    # at least 3 warm-up steps, whatever is asked
    assert line["steps"] == 2 and line["warmup"] == 3 and line["n_gpus"] == 1
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["value"] == line["value"] and cb["cores"] >= 1
    assert "24^3" in cb["sample"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["unit"] == "GLUPS"
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
