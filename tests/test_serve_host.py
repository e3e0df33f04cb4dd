"""Host logic of the batched and served workloads, without a GPU: the solve
distribution of the batched ensemble, the Poisson arrival stream and the
latency summary of lbswim.serve."""
import math
import time

import numpy as np

from lbswim import serve


def test_solve_distribution_ranges():
    # shapes from the ensemble list, tau ~ U[0.6, 1.5], swimmers log-uniform
    # in [1, 512] with P ~ U[1e-4, 1e-3] and alpha ~ U[0, 0.05], tracers in
    # [0, 4096], steps log-uniform in the requested range
    rng = np.random.default_rng(1)
    specs = [serve.draw_spec(rng, steps_range=(100, 5000)) for _ in range(4000)]
    assert {s.shape for s in specs} == set(serve.ENSEMBLE_SHAPES)
    tau = np.array([s.tau for s in specs])
    assert tau.min() >= 0.6 and tau.max() < 1.5
    nsw = np.array([s.nsw for s in specs])
    assert nsw.min() >= 1 and nsw.max() <= 512
    # log-uniform: the median of log(n) sits near log(512) / 2
    assert abs(np.median(np.log(nsw)) - math.log(512.0) / 2) < 0.25
    P = np.array([s.P for s in specs])
    assert P.min() >= 1e-4 and P.max() < 1e-3
    alpha = np.array([s.alpha for s in specs])
    assert alpha.min() >= 0.0 and alpha.max() < 0.05
    ntr = np.array([s.ntr for s in specs])
    assert ntr.min() >= 0 and ntr.max() <= 4096 and abs(ntr.mean() - 2048) < 100
    steps = np.array([s.steps for s in specs])
    assert steps.min() >= 100 and steps.max() <= 5000
    assert len({s.seed for s in specs}) > 3990


def test_poisson_trace_is_seeded_ordered_and_at_rate():
    rate, duration = 200.0, 30.0
    a = serve.poisson_trace(np.random.default_rng(11), rate, duration)
    b = serve.poisson_trace(np.random.default_rng(11), rate, duration)
    assert [t for t, _ in a] == [t for t, _ in b]
    assert [s.seed for _, s in a] == [s.seed for _, s in b]
    times = np.array([t for t, _ in a])
    assert np.all(np.diff(times) > 0) and times[-1] < duration
    n = len(a)
    assert abs(n - rate * duration) < 5 * math.sqrt(rate * duration)
    assert {s.shape for _, s in a} <= set(serve.SERVING_SHAPES)


def test_summary_nearest_rank_percentiles():
    done = [{"latency": float(x)} for x in np.random.default_rng(2).permutation(100) + 1]
    s = serve.summary({"done": done, "unfinished": 7, "updates": 3e9, "wall": 2.0})
    assert s["p50_s"] == 50.0 and s["p99_s"] == 99.0
    assert s["completed"] == 100 and s["unfinished"] == 7
    assert s["glups"] == 1.5 and s["wall_s"] == 2.0
    empty = serve.summary({"done": [], "unfinished": 3, "updates": 0, "wall": 1.0})
    assert empty["p50_s"] is None and empty["p99_s"] is None and empty["completed"] == 0


def test_device_bytes_grow_with_size_and_storage():
    small = serve.Spec((16, 16, 16), 0.8, 10, 1e-3, 0.01, 100, 1)
    large = serve.Spec((128, 128, 128), 0.8, 10, 1e-3, 0.01, 100, 1)
    assert large.device_bytes() > small.device_bytes()
    b64, b32, b16 = (large.device_bytes(p) for p in ("f64", "f32", "bf16"))
    assert b64 > b32 > b16
    # the distributions dominate: two f buffers of 15 values per site
    assert b32 > 2 * 15 * 4 * large.sites


# ---- the serving loop's fault handling, with a fake GPU ----------------------
class _FakeEnsemble:
    """Stands in for the batched stepper: records memberships and steps, each
    Step call taking `delay` seconds."""

    def __init__(self, delay=0.0):
        self.members, self.steps, self.delay = [], 0, delay

    def set_members(self, members):
        self.members = list(members)

    def autotune(self):
        pass

    def Step(self, k, limits=None):
        assert self.members
        assert limits is None or (len(limits) == len(self.members) and max(limits) <= k)
        self.steps += k
        if self.delay:
            time.sleep(self.delay)


class _FakeBuild:
    """Stands in for build_solve; `fail` maps a request seed to the number of
    allocation failures (LBSWIM_ENOMEM) its first builds raise."""

    def __init__(self, fail=None):
        self.fail = dict(fail or {})
        self.calls = 0

    def __call__(self, spec, precision, lattice=None):
        from lbswim import _lib
        self.calls += 1
        if self.fail.get(spec.seed, 0) > 0:
            self.fail[spec.seed] -= 1
            raise _lib.LbswimError(-3, "cudaMalloc: out of memory (injected)")
        return (lattice or ("lattice", spec.seed), None, None)


def _trace(n, steps=40, shape=(16, 16, 16)):
    return [(0.0, serve.Spec(shape, 0.8, 4, 1e-3, 0.01, 8, 100 + i, steps)) for i in range(n)]


def _outcomes(res, n):
    seen = [d["index"] for d in res["done"]] + [r["index"] for r in res["rejected"]] + \
        [c["index"] for c in res["cancelled"]]
    assert sorted(seen) == list(range(n)), seen  # every request exactly once


def test_malformed_and_oversized_requests_are_rejected_and_the_loop_goes_on():
    trace = _trace(4)
    trace[1] = (0.0, serve.Spec((16, 0, 16), 0.8, 4, 1e-3, 0.01, 8, 7, 40))       # bad shape
    trace[2] = (0.0, serve.Spec((16, 16, 16), 0.8, 4, 1e-3, 0.01, 8, 8, 0))        # no steps
    big = serve.Spec((512, 512, 512), 0.8, 4, 1e-3, 0.01, 8, 9, 40)
    trace.append((0.0, big))
    budget = 3 * trace[0][1].device_bytes()
    srv = serve.Server(budget, chunk=16, build=_FakeBuild(), ensemble=_FakeEnsemble())
    res = srv.run(trace, duration=5.0, drain=True)
    _outcomes(res, len(trace))
    why = {r["index"]: r["reason"] for r in res["rejected"]}
    assert set(why) == {1, 2, 4}
    assert "shape" in why[1] and "step" in why[2] and "budget" in why[4]
    assert sorted(d["index"] for d in res["done"]) == [0, 3]


def test_allocation_failures_wait_for_memory_or_reject():
    trace = _trace(3)
    budget = 3 * trace[0][1].device_bytes()
    # request 1 fails twice while request 0 runs: it waits, then runs
    build = _FakeBuild({trace[1][1].seed: 2})
    srv = serve.Server(budget, chunk=8, build=build, ensemble=_FakeEnsemble())
    res = srv.run(trace, duration=5.0, drain=True)
    _outcomes(res, 3)
    assert sorted(d["index"] for d in res["done"]) == [0, 1, 2] and not res["rejected"]
    # alone, with nothing to free, a request whose allocation keeps failing is rejected
    srv = serve.Server(budget, chunk=8, build=_FakeBuild({trace[0][1].seed: 99}),
                       ensemble=_FakeEnsemble())
    res = srv.run(trace[:1], duration=5.0, drain=True)
    assert res["rejected"] == [{"index": 0, "reason": "device allocation failed"}]


def test_cancelled_requests_leave_the_queue_and_the_batch():
    trace = _trace(5, steps=4000)
    trace[4] = (0.3, trace[4][1])  # arrives late
    budget = 2 * trace[0][1].device_bytes()  # two run, the rest queue
    srv = serve.Server(budget, chunk=64, build=_FakeBuild(), ensemble=_FakeEnsemble(0.002))
    # 0 is running at 0.03 s (63 chunks of 2 ms each), 3 still queued
    res = srv.run(trace, duration=10.0, drain=True, cancel={0: 0.03, 3: 0.03, 4: 0.1})
    _outcomes(res, 5)
    where = {c["index"]: c["where"] for c in res["cancelled"]}
    assert where == {0: "batch", 3: "queue", 4: "before arrival"}
    assert sorted(d["index"] for d in res["done"]) == [1, 2]
