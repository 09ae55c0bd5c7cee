"""The bench's replica logic across ranks, on CPU with the gloo backend
(world size 2, rendezvous on 127.0.0.1): the timed duration is the maximum over
ranks, the whole-job value counts every rank's units, and only rank 0 reports."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        elapsed = 10.0 + 5.0 * rank  # rank 1 is the slow one
        slowest = bench.max_over_ranks(elapsed, dist, "cpu")
        value = bench.job_throughput(world, 1000, slowest)
        dist.barrier()
        q.put((rank, slowest, value, bench.reports(rank)))
    finally:
        dist.destroy_process_group()


def test_two_rank_replicas_gloo():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    assert [g[0] for g in got] == [0, 1]
    for rank, slowest, value, reports in got:
        assert slowest == 15.0                  # max over ranks
        assert value == pytest.approx(2 * 1000 / 15.0)
        assert reports == (rank == 0)


def test_single_process_without_dist():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.5, None, "cpu") == 3.5
    assert bench.job_throughput(1, 10, 2.0) == 5.0
