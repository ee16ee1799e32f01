"""bench.py's multi-GPU form is N independent replicas (no data-path collective):
the job's time is the slowest rank's and its rate counts every rank's work.
Checked with two gloo ranks on the CPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    t = bench.max_over_ranks(1.5 + rank, dist, "cpu")
    out[rank] = (t, bench.replica_rate(1000, world, t))
    dist.destroy_process_group()


def test_two_replicas_take_the_slowest_time_and_count_both():
    world = 2
    with mp.get_context("spawn").Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_rank, args=(world, _free_port(), out), nprocs=world, join=True)
        res = dict(out)
    for rank in range(world):
        t, rate = res[rank]
        assert t == 2.5 and rate == pytest.approx(2 * 1000 / 2.5)
    import bench

    assert bench.max_over_ranks(3.0) == 3.0
