"""Independent solves shared out over GPUs (lbswim.shard): the assignment is
deterministic and balanced, and two gloo ranks on the CPU serving their shares
of one stream (fake GPU) finish every request exactly once."""
import os
import socket

import numpy as np
import pytest

from lbswim import serve, shard


def test_assignment_is_deterministic_and_balanced():
    rng = np.random.default_rng(5)
    specs = [serve.draw_spec(rng, steps_range=(100, 5000)) for _ in range(512)]
    a = shard.assign(specs, 4)
    assert a == shard.assign(specs, 4)
    load = [sum(shard.work_of(s) for s, r in zip(specs, a) if r == k) for k in range(4)]
    assert max(load) <= 1.05 * min(load)
    # a rank with twice the capacity takes about twice the work
    b = shard.assign(specs, 2, capacity=[2.0, 1.0])
    l2 = [sum(shard.work_of(s) for s, r in zip(specs, b) if r == k) for k in range(2)]
    assert 1.8 < l2[0] / l2[1] < 2.2
    assert shard.assign(specs, 1) == [0] * len(specs)
    with pytest.raises(ValueError):
        shard.assign(specs, 2, capacity=[1.0])


def test_stream_assignment_depends_on_the_trace_only():
    trace = serve.poisson_trace(np.random.default_rng(2), 200.0, 5.0)
    a = shard.assign_stream(trace, 3)
    assert a == shard.assign_stream(trace, 3) and set(a) == {0, 1, 2}
    assert sorted(i for k in range(3) for i, _ in shard.mine(trace, a, k)) == \
        list(range(len(trace)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from test_serve_host import _FakeBuild, _FakeEnsemble
    rng = np.random.default_rng(9)
    trace = [(0.001 * i, serve.draw_spec(rng, serve.ENSEMBLE_SHAPES, (10, 60)))
             for i in range(40)]
    ranks = shard.assign_stream(trace, world)
    local = shard.mine(trace, ranks, rank)
    sub = [(a, s) for _, (a, s) in local]
    srv = serve.Server(1 << 40, chunk=16, build=_FakeBuild(), ensemble=_FakeEnsemble())
    res = srv.run(sub, duration=10.0, drain=True)
    # back to global trace indices
    glob = [i for i, _ in local]
    for d in res["done"]:
        d["index"] = glob[d["index"]]
    res.pop("kept")
    merged = shard.merge_served(shard.gather_objects(res, world))
    if rank == 0:
        q.put(sorted(d["index"] for d in merged["done"]))
    dist.destroy_process_group()


def test_two_gloo_ranks_serve_every_request_exactly_once():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got == list(range(40))
