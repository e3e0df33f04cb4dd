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
    srv = serve.Server(budget, chunk=16, autotune=False, readback=True)
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
        # the result the server handed back is that state
        got = next(d["result"] for d in res["done"] if d["index"] == i)
        assert np.array_equal(got["u"].reshape(3, -1), b["u"]) and got["time_step"] == spec.steps
        assert np.array_equal(got["sw_r"], b["sw_r"]) and np.array_equal(got["sw_n"], b["sw_n"])
        if tr is not None:
            assert np.array_equal(got["tr_r"], b["tr_r"])


def test_summary_reports_latency_percentiles():
    from lbswim import serve
    res = {"done": [{"latency": x} for x in np.linspace(1.0, 100.0, 100)], "updates": 10**9,
           "wall": 2.0, "unfinished": 3}
    s = serve.summary(res)
    assert s["completed"] == 100 and s["unfinished"] == 3
    assert s["p50_s"] == 50.0 and s["p99_s"] == 99.0 and s["glups"] == 0.5


def test_device_initial_state_is_seeded_and_precision_independent():
    from lbswim import lb, swimmers, tracers
    states = []
    for precision in ("f64", "f32"):
        lat = lb.Lattice(20, 12, 16, 0.9, 0.9, precision=precision)
        lat.init_random(77)
        sw = swimmers.Array(50, swimmers.CommonParams())
        sw.init_random(lat, 77)
        tr = tracers.Array(80)
        tr.init_random(lat, 78)
        lat.rho.D2H()
        sw.D2H()
        tr.D2H()
        states.append((lat.rho.data.copy(), sw.r.data.copy(), sw.n.data.copy(), tr.r.data.copy()))
    (rho64, r64, n64, t64), (rho32, r32, n32, t32) = states
    assert np.all((rho64 >= 1.0) & (rho64 < 1.001))
    assert np.abs(rho32 - rho64).max() < 1e-9
    assert np.array_equal(r64, r32) and np.array_equal(n64, n32) and np.array_equal(t64, t32)
    assert np.allclose((n64 ** 2).sum(axis=0), 1.0, atol=1e-14)
    assert np.all(r64 >= 0) and np.all(r64[0] < 20) and np.all(r64[1] < 12) and np.all(r64[2] < 16)
