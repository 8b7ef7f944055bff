"""Sharding of independent units over ranks, on CPU (gloo, world size 2).

Reactors of a batch (and tubes of an uneven set) do not interact, so ranks
take contiguous cost-balanced ranges and gather once at the end; the union
of the ranks' results must equal the single-rank result bit for bit. The
per-rank work here is the oracle's reactor batch (CPU), standing in for a
rank's GPU batch call; the partition and the gather are the path's own.
"""
import os
import sys
from pathlib import Path

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))

from fortrancfd_gb300.shard import my_range, partition  # noqa: E402


def test_partition_covers_in_order_and_balances():
    rng = np.random.default_rng(0)
    costs = rng.uniform(2000, 50000, 256)  # cells of 256 uneven tubes
    for world in (1, 2, 3, 4, 8):
        parts = partition(costs, world)
        assert parts[0][0] == 0 and parts[-1][1] == len(costs)
        assert all(parts[r][1] == parts[r + 1][0] for r in range(world - 1))
        share = np.array([costs[a:b].sum() for a, b in parts])
        # no rank holds more than its share plus one unit
        assert share.max() <= costs.sum() / world + costs.max()
    assert partition([], 3) == [(0, 0)] * 3
    assert partition([1.0, 1.0], 4)[-1] == (2, 2)
    assert partition([0.0] * 10, 2) == [(0, 5), (5, 10)]
    with pytest.raises(ValueError):
        partition([1.0, -1.0], 2)


def _batch(n):
    from fortrancfd_gb300 import configs

    rho, dt, yiT, _ = configs.reactor_batch(n, seed=21)
    return rho, dt * 0.1, yiT


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, str(ROOT))
    sys.path.insert(0, str(ROOT / "tests"))
    from oracle_ctypes import Oracle

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        rho, dt, yiT = _batch(12)
        a, b = my_range(np.ones(len(rho)), rank, world)
        y, fails, _ = Oracle().reactor_batch(rho[a:b], dt[a:b], yiT[a:b], 1e-6, 1e-14, nthreads=1)
        parts = [None] * world
        dist.all_gather_object(parts, (a, b, y, fails))
        if rank == 0:
            q.put(parts)
    finally:
        dist.destroy_process_group()


def test_two_ranks_union_equals_single_rank():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29700 + os.getpid() % 1000
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    parts = q.get(timeout=300)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    sys.path.insert(0, str(ROOT / "tests"))
    from oracle_ctypes import Oracle

    rho, dt, yiT = _batch(12)
    whole, fails, _ = Oracle().reactor_batch(rho, dt, yiT, 1e-6, 1e-14, nthreads=1)
    assert fails == 0 and all(p[3] == 0 for p in parts)
    union = np.concatenate([p[2] for p in sorted(parts, key=lambda p: p[0])])
    assert [p[:2] for p in parts] == [(0, 6), (6, 12)]
    assert np.array_equal(union, whole)
