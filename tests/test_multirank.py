"""The N > 1 path of bench.py on CPU: world size 2 over gloo.

Each rank runs its own replica of the tube (no data-path collective); the
job's time is the max over ranks and its value counts every rank's cells.
The reference arm runs on rank 0 only; other ranks return without work.
"""
import os
import sys
from pathlib import Path

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parents[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, str(ROOT))
    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        r, w, local = bench.dist_env()
        t = bench.max_over_ranks(1.0 + rank, w)       # rank 1 is the slow one
        v = bench.job_value(20000, 32, w, t)
        dist.barrier()
        # the reference arm: rank 0 alone works; other ranks return at once
        skipped = bench.reference_arm(None, r, w) is None if r != 0 else None
        q.put((r, w, local, t, v, skipped))
    finally:
        dist.destroy_process_group()


def test_two_ranks_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[0] for o in out] == [0, 1]
    for r, w, local, t, v, _ in out:
        assert w == 2 and local == r
        assert t == 2.0                                  # max over ranks
        assert v == pytest.approx(20000 * 32 * 2 / 2.0)  # all ranks' cells over the slowest time
    assert out[1][5] is True


def test_single_rank_is_identity():
    sys.path.insert(0, str(ROOT))
    import bench

    assert bench.max_over_ranks(3.5, 1) == 3.5
    assert bench.job_value(100, 10, 1, 2.0) == 500.0
