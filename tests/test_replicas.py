"""Replicas on several ranks (CPU, gloo, world size 2): the benchmark's
whole-job throughput takes the slowest rank's time (max over ranks) and
counts the units of every rank; ranks run the same seeded workload."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
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
        elapsed = 10.0 + 5.0 * rank                     # rank 1 is the slow one
        slowest = bench.max_over_ranks(elapsed, dist, "cpu")
        rate = bench.whole_job_rate(1_000_000, world, 4, slowest)
        out[rank] = (slowest, rate)
    finally:
        dist.destroy_process_group()


def test_two_replicas_report_the_slowest_rank():
    port = _free_port()
    manager = mp.get_context("spawn").Manager()
    out = manager.dict()
    mp.spawn(_rank, args=(2, port, out), nprocs=2, join=True)
    assert out[0] == out[1]
    slowest, rate = out[0]
    assert slowest == 15.0
    # 2 ranks x 4 steps x 1e6 units in 15 ms
    assert abs(rate - 2 * 4 * 1e6 / 0.015 / 1e6) < 1e-6


def test_single_rank_needs_no_process_group():
    assert bench.max_over_ranks(3.5, None, "cpu") == 3.5
    assert bench.whole_job_rate(2e6, 1, 2, 4.0) == pytest.approx(2 * 2e6 / 0.004 / 1e6)
