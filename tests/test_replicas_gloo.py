"""The multi-rank bench path (replicas, no data-path collective): the whole-job rate is every
rank's queries over the slowest rank's time. Two gloo ranks on the CPU."""
import os

import pytest
import torch.multiprocessing as mp


def _rank(rank, world, port, q):
    import torch.distributed as dist

    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        slowest = bench.max_over_ranks(1.0 + rank, dist, "cpu")  # rank 1 is the slower one
        q.put((rank, slowest, bench.whole_job_rate(1000, 10, world, slowest)))
    finally:
        dist.destroy_process_group()


def test_two_replicas_take_the_slowest_rank():
    import socket

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in procs)
    assert [g[1] for g in got] == [2.0, 2.0]
    assert all(g[2] == pytest.approx(1000 * 10 * 2 / 2.0) for g in got)


def test_single_process_is_unchanged():
    import bench

    assert bench.max_over_ranks(3.5, None, "cpu") == 3.5
    assert bench.whole_job_rate(10000, 20, 1, 0.064) == pytest.approx(3125000.0)
