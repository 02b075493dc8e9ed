"""Multi-process (gloo, world size 2, CPU) check of bench.py's replica
aggregation: each rank times its own replica, the job time is the max over
ranks, the job rate counts every rank's steps, and the replicas draw
different particles."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, times, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    t = bench.max_over_ranks(times[rank], world, "cpu")
    out[rank] = (t, bench.job_rate(world, 10, t), bench.replica_seed(rank))
    dist.barrier()
    dist.destroy_process_group()


def test_two_ranks_max_and_rate():
    import torch.multiprocessing as mp
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    times = [0.25, 0.4]
    mp.spawn(_worker, args=(2, _free_port(), times, out), nprocs=2, join=True)
    for r in (0, 1):
        t, rate, _ = out[r]
        assert t == pytest.approx(0.4)
        assert rate == pytest.approx(2 * 10 / 0.4)
    assert out[0][2] != out[1][2]


def test_one_rank_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(1.5, 1, "cpu") == 1.5
    assert bench.job_rate(1, 4, 2.0) == 2.0
