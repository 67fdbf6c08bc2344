"""Splitting a batch of pairs across GPUs (one process per GPU).

Pairs are independent, so a batch shards with no exchange on the data path:
each rank takes a contiguous range of pairs whose estimated cost is about a
1/world share of the total (ConvexHull pairs cost in proportion to the hull
points the support-point arg-max scans; analytic pairs a constant), runs it on
its own GPU, and the host gathers the outputs in pair order.  The shape table
and hull points stay whole on every rank (pairs index into them).
"""
from __future__ import annotations

import numpy as np

from .shapes import PairBatch

ANALYTIC_COST = 64.0  # in hull-point units: a GJK/EPA of analytic shapes


def pair_cost(batch: PairBatch) -> np.ndarray:
    """Estimated relative cost of each pair."""
    n = batch.shapes["hull_n"].astype(np.float64)
    hull = batch.shapes["kind"] == 5
    per_shape = np.where(hull, n, 0.0)
    return ANALYTIC_COST + per_shape[batch.g1] + per_shape[batch.g2]


def shard_ranges(cost: np.ndarray, world: int) -> list[tuple[int, int]]:
    """Contiguous [start, end) ranges, one per rank, balancing the summed cost."""
    if world < 1:
        raise ValueError("world must be >= 1")
    n = len(cost)
    cum = np.concatenate([[0.0], np.cumsum(cost, dtype=np.float64)])
    cuts = [0]
    for r in range(1, world):
        cuts.append(int(np.searchsorted(cum, cum[-1] * r / world, side="left")))
    cuts.append(n)
    cuts = np.maximum.accumulate(np.minimum(np.asarray(cuts), n))
    return [(int(cuts[r]), int(cuts[r + 1])) for r in range(world)]


def shard(batch: PairBatch, world: int, rank: int) -> tuple[PairBatch, tuple[int, int]]:
    """This rank's pairs (and their range in the batch)."""
    a, b = shard_ranges(pair_cost(batch), world)[rank]
    return batch.subset(np.arange(a, b)), (a, b)


def gather(local: dict, rng: tuple[int, int], n_total: int, group=None) -> dict | None:
    """Gathers per-rank numpy outputs (arrays indexed by pair) into pair order on
    rank 0 through torch.distributed (any backend that supports objects)."""
    import torch.distributed as dist
    world = dist.get_world_size(group)
    parts = [None] * world
    dist.all_gather_object(parts, (rng, local), group=group)
    if dist.get_rank(group) != 0:
        return None
    out = {}
    for (a, b), d in parts:
        for k, v in d.items():
            if k not in out:
                out[k] = np.zeros((n_total,) + v.shape[1:], v.dtype)
            out[k][a:b] = v
    return out
