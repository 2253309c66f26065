"""The bench's multi-GPU path runs replicas (one grid per rank, no data-path
collective): the job's time is the slowest rank's and the throughput is the
sum over ranks.  Checked with two gloo ranks on the CPU."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = bench.slowest_rank_ms(10.0 + 2.5 * rank, dist, "cpu")
        q.put((rank, ms, bench.replicas_value(4096 * 4096, 200, ms, world)))
    finally:
        dist.destroy_process_group()


def test_replicas_take_the_slowest_rank():
    import socket

    import torch.multiprocessing as mp

    with socket.socket() as sck:
        sck.bind(("127.0.0.1", 0))
        port = sck.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for pr in procs:
        pr.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for pr in procs:
        pr.join(timeout=60)
        assert pr.exitcode == 0
    assert [o[1] for o in out] == [12.5, 12.5]
    want = 2 * 4096 * 4096 * 200 / 12.5e-3
    assert all(abs(o[2] - want) <= 1e-9 * want for o in out)


def test_one_rank_needs_no_collective():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.slowest_rank_ms(7.25, None, "cpu") == 7.25
    assert bench.replicas_value(100, 10, 1.0, 1) == 1e6
