"""The multi-GPU mode of bench.py is independent replicas (the solve path has no exchange step):
each rank runs its own box and the ranks only share the clock.  This checks that host logic on
CPU with two gloo ranks: every rank sees the slowest rank's time, and the whole-job rate counts
the units of all ranks over that time."""
import os
import socket

import pytest
import torch.multiprocessing as mp

import bench


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, times, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        t = bench.max_over_ranks(times[rank], world, "cpu")
        out[rank] = (t, bench.replica_rate(1000, 10, world, t))
    finally:
        dist.destroy_process_group()


def test_two_replicas_share_the_slowest_time():
    world = 2
    times = [0.25, 0.40]
    with mp.get_context("spawn").Manager() as m:   # no fork of a multi-threaded test process
        out = m.dict()
        mp.spawn(_rank, args=(world, _free_port(), times, out), nprocs=world, join=True)
        res = dict(out)
    for r in range(world):
        t, rate = res[r]
        assert t == pytest.approx(0.40)
        assert rate == pytest.approx(1000 * 10 * world / 0.40)


def test_single_rank_needs_no_process_group():
    assert bench.max_over_ranks(0.3, 1, "cpu") == pytest.approx(0.3)
    assert bench.replica_rate(9437184, 50, 1, 0.01) == pytest.approx(9437184 * 50 / 0.01)
