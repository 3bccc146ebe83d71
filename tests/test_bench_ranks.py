"""bench.py's multi-rank glue on CPU: world_size 2 over gloo, each rank with
its own step time; the job time is the slowest rank's and the throughput
counts both ranks' batches (weak scaling, no data-path collective)."""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

import bench


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = 100.0 + 50.0 * rank  # rank 1 is slower
        worst = bench.max_over_ranks(ms, dist, "cpu")
        out[rank] = (worst, bench.job_throughput(1000, worst, world))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_step():
    world = 2
    out = mp.Manager().dict()
    mp.spawn(_rank, args=(world, _free_port(), out), nprocs=world, join=True)
    for r in range(world):
        worst, thr = out[r]
        assert worst == 150.0
        assert thr == pytest.approx(2 * 1000 / 0.150)


def test_single_process_needs_no_group():
    assert bench.max_over_ranks(42.0, None, "cpu") == 42.0
    assert bench.job_throughput(500, 250.0, 1) == pytest.approx(2000.0)
