"""Partition of independent work units (reactors of a batch, tubes of an
uneven set, cells of a chemistry step) over the ranks of a job.

The reference splits its one tube into contiguous per-rank block ranges
(SRC/parallel.f90:66-83) and exchanges halos between them. Units that do
not interact need no exchange at all: each rank takes one contiguous range
of units whose summed cost is as close as possible to an equal share, works
on it alone, and the results are gathered once at the end.
"""
from __future__ import annotations

from typing import List, Sequence, Tuple

import numpy as np


def partition(costs: Sequence[float], world: int) -> List[Tuple[int, int]]:
    """Contiguous ranges [a, b), one per rank, covering all units in order:
    rank r's range ends at the first unit where the running cost reaches
    (r + 1) / world of the total (ties towards the earlier boundary), so
    every rank gets a near-equal share of the cost and no unit is split.
    Deterministic; empty ranges only when there are fewer units than
    ranks."""
    c = np.asarray(costs, dtype=np.float64)
    n = len(c)
    if world < 1:
        raise ValueError("world must be >= 1")
    if np.any(c < 0) or not np.all(np.isfinite(c)):
        raise ValueError("costs must be finite and non-negative")
    if n == 0:
        return [(0, 0)] * world
    pref = np.concatenate([[0.0], np.cumsum(c)])
    total = pref[-1]
    bounds = [0]
    for r in range(1, world):
        if total > 0:
            b = int(np.searchsorted(pref, total * r / world, side="left"))
        else:
            b = (n * r) // world
        bounds.append(min(max(b, bounds[-1]), n))
    bounds.append(n)
    return [(bounds[r], bounds[r + 1]) for r in range(world)]


def my_range(costs: Sequence[float], rank: int, world: int) -> Tuple[int, int]:
    """This rank's range of partition(costs, world)."""
    return partition(costs, world)[rank]
