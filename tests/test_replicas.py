"""Replica timing across ranks, on CPU with gloo.

The cylinder bench runs one independent replica per rank (no collective on the
data path); the only exchange is the timing, where the job's time is the
slowest rank's.  This runs that reduction with two gloo ranks on 127.0.0.1.
"""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, times, out):
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    import bench

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        out.put((rank, bench.max_over_ranks(times[rank], world, device="cpu")))
    finally:
        dist.destroy_process_group()


def test_one_rank_is_its_own_time():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.max_over_ranks(12.5, 1) == 12.5


def test_two_ranks_agree_on_the_slowest():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    times = [3.25, 7.75]
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_rank, args=(r, 2, port, times, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got == {0: 7.75, 1: 7.75}
