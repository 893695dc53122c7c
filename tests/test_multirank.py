"""The multi-GPU path of the benchmark on CPU: two gloo ranks (127.0.0.1).
Every rank runs its own replica of the workload; the job's time is the
largest rank time and the job's GB/s counts every rank's bytes (weak
scaling, no collective in the data path)."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

import bench


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, times, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = bench.max_over_ranks(torch, dist, times[rank], device="cpu")
        out[rank] = (ms, bench.job_gbs(1 << 30, world, ms))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("times", [(2.0, 3.5), (7.25, 1.0)])
def test_two_ranks_take_the_slowest_rank(times):
    world = 2
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(world, _free_port(), list(times), out), nprocs=world, join=True)
        res = dict(out)
    slow = max(times)
    for r in range(world):
        ms, gbs = res[r]
        assert ms == slow
        assert abs(gbs - (1 << 30) * world / (slow / 1e3) / 1e9) < 1e-9


def test_single_process_keeps_its_own_time():
    assert bench.max_over_ranks(torch, None, 4.5) == 4.5
    assert bench.job_gbs(2e9, 1, 1000.0) == 2.0
