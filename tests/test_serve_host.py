"""Host logic of the batched and served workloads, without a GPU: the solve
distribution of the batched ensemble, the Poisson arrival stream and the
latency summary of lbswim.serve."""
import math

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
