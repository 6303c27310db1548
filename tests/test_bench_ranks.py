"""bench.py's multi-GPU aggregation on CPU: two gloo ranks, each with its own
timing, agree on the slowest rank's time, and the whole-job rate counts the
units of every rank (replicas, weak scaling)."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = 100.0 + 50.0 * rank  # rank 1 is the slower one
    m = bench.max_over_ranks(ms, dist, "cpu")
    out[rank] = (m, bench.whole_job_rate(200, world, m / 1000.0))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_agree_on_the_slowest_time():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    world, port = 2, _free_port()
    with mp.get_context("spawn").Manager() as man:  # no fork of a process that may hold OpenMP threads
        out = man.dict()
        mp.start_processes(_rank, args=(world, port, out), nprocs=world, join=True, start_method="spawn")
        res = dict(out)
    assert res[0][0] == res[1][0] == 150.0
    assert res[0][1] == res[1][1] == pytest.approx(200 * 2 / 0.150)


def test_single_rank_needs_no_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(12.5) == 12.5
    assert bench.whole_job_rate(300, 1, 0.5) == 600.0
