"""The N-GPU form of bench.py runs independent replicas: the only traffic
between ranks is the barrier and the max-over-ranks of the timings, and rank 0
alone prints.  Exercised here as two gloo ranks on the CPU."""
import io
import os
import sys
import contextlib

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank,
                           world_size=world)
    got = bench.max_over_ranks(1.5 + rank, world)
    buf = io.StringIO()
    with contextlib.redirect_stdout(buf):
        bench.emit({"rank": rank, "max": got}, rank)
    dist.barrier()
    dist.destroy_process_group()
    out.put((rank, got, buf.getvalue()))


def test_two_gloo_ranks_reduce_max_and_print_once():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [2.5, 2.5]
    assert res[0][2].strip() == '{"rank": 0, "max": 2.5}'
    assert res[1][2] == ""
