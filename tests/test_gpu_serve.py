"""Serving: continuous batching under an HBM budget.

Solves that arrive while others run join the batch; each finished solve is
the same, bit for bit, as that solve run alone through System.Step with the
same slab shape.
"""
import numpy as np
import pytest

from gpu_harness import snapshot

pytestmark = pytest.mark.gpu


def test_solves_in_the_mix_equal_alone():
    from lbswim import serve
    from lbswim.System import System
    rng = np.random.default_rng(3)
    shapes = [(16, 16, 16), (24, 24, 24), (32, 32, 64)]
    trace = []
    t = 0.0
    for i in range(6):
        spec = serve.draw_spec(rng, shapes, (20, 90))
        trace.append((t, spec))
        t += 0.002
    budget = sum(s.device_bytes() for _, s in trace[:4])  # two must wait for memory
    srv = serve.Server(budget, chunk=16, autotune=False)
    res = srv.run(trace, duration=60.0, drain=True, keep=set(range(len(trace))))
    assert len(res["done"]) == len(trace) and res["unfinished"] == 0
    assert max(d["queue"] for d in res["done"]) > 0.0  # someone waited for memory
    for i, (_, spec) in enumerate(trace):
        lat, sw, tr = serve.build_solve(spec)
        mixed = res["kept"][i]
        lat.tile = mixed[0].tile
        system = System(lat)
        system.AddThing(sw)
        if tr is not None:
            system.AddThing(tr)
        system.Step(spec.steps)
        a, b = snapshot(*mixed), snapshot(lat, sw, tr)
        for k in a:
            assert np.array_equal(a[k], b[k]), (i, k)


def test_summary_reports_latency_percentiles():
    from lbswim import serve
    res = {"done": [{"latency": x} for x in np.linspace(1.0, 100.0, 100)], "updates": 10**9,
           "wall": 2.0, "unfinished": 3}
    s = serve.summary(res)
    assert s["completed"] == 100 and s["unfinished"] == 3
    assert s["p50_s"] == 50.0 and s["p99_s"] == 99.0 and s["glups"] == 0.5
