"""The multi-GPU path is replicas only: each rank runs its own allocator and
the job's throughput is all ranks' work over the slowest rank's time. The
host-side reduction is exercised here with two gloo ranks on the CPU."""
from __future__ import annotations

import os
import socket
import sys
from pathlib import Path

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

REPO = Path(__file__).resolve().parent.parent


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out):
    sys.path.insert(0, str(REPO))
    import bench

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        slowest = bench.barrier_max(torch, world, 10.0 + 5.0 * rank, device="cpu")
        out[rank] = (slowest, bench.replica_throughput(1000, 4, world, slowest))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_time():
    world = 2
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank_main, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    assert res[0][0] == res[1][0] == 15.0
    # 2 replicas x 1000 units x 4 steps over the slowest 15 ms
    assert res[0][1] == pytest.approx(2 * 1000 * 4 / 0.015)


def test_single_replica_needs_no_process_group():
    sys.path.insert(0, str(REPO))
    import bench

    assert bench.barrier_max(torch, 1, 3.5) == 3.5
    assert bench.replica_throughput(10, 2, 1, 1000.0) == pytest.approx(20.0)
