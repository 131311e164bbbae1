"""bench.py --gpus N runs N independent replicas (the step does not shard):
the timing helpers take the barrier and the maximum over ranks. Checked with
two gloo ranks on the CPU."""

import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, out):
    import torch
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        bench.barrier(dist, torch)
        value = bench.max_over_ranks(1.5 + rank, dist, torch)
        total = world * 100 * 10 / value  # cells x steps over the slowest rank's time
        out.put((rank, value, total))
    finally:
        dist.destroy_process_group()


def test_max_over_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [v for _, v, _ in got] == [2.5, 2.5]
    assert all(abs(t - 2 * 1000 / 2.5) < 1e-9 for _, _, t in got)


def test_single_rank_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.25, None, None) == 3.25
    bench.barrier(None, None)
