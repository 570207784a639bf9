"""bench.py's multi-rank bookkeeping (replicas: a barrier, the maximum of the timed
totals, the whole-job aggregate) with two gloo ranks on the CPU."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, q):
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        bench.sync_ranks(world)
        local_ms = 100.0 + 25.0 * rank  # the second rank is slower
        m = bench.max_over_ranks(local_ms, world, device="cpu")
        q.put((rank, m, bench.aggregate_mrays(world, 1_000_000, 10, m)))
    finally:
        dist.destroy_process_group()


def test_two_ranks_take_the_slowest_time():
    import socket

    import torch.multiprocessing as mp

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    for rank, m, agg in got:
        assert m == 125.0
        # 2 ranks x 1M rays x 10 steps in 0.125 s
        assert agg == pytest.approx(2 * 1_000_000 * 10 / 0.125 / 1e6)


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench

    bench.sync_ranks(1)
    assert bench.max_over_ranks(7.5, 1) == 7.5
    assert bench.aggregate_mrays(1, 100, 10, 1000.0) == pytest.approx(0.001)
