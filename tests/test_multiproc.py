"""Replica runs across ranks, on CPU with gloo (world size 2).

The path does not exchange data between GPUs: each rank renders its own
frames and bench.py combines the slowest rank's time with the summed work.
"""
from __future__ import annotations

import os
import socket
import sys
from pathlib import Path

import pytest
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank: int, world: int, port: int, q):
    sys.path.insert(0, str(ROOT))
    import torch.distributed as dist

    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r "took" 100 + 50 r ms for 1000 (r + 1) samples and 10 (r + 1) rays
        res = bench.aggregate_ranks(100.0 + 50.0 * rank, 1000 * (rank + 1), 10 * (rank + 1), dist, "cpu")
        ref = bench.reference_arm(None, rank, world) if rank != 0 else "rank0"
        q.put((rank, res, ref))
    finally:
        dist.destroy_process_group()


def test_replica_aggregation_two_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = {}
    for _ in procs:
        rank, res, ref = q.get(timeout=120)
        out[rank] = (res, ref)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank in (0, 1):
        ms, samples, rays = out[rank][0]
        assert ms == 150.0 and samples == 3000.0 and rays == 30.0
    assert out[1][1] is None  # the reference arm does no work off rank 0


def test_single_rank_passthrough():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.aggregate_ranks(12.5, 7, 3, None) == (12.5, 7.0, 3.0)
