"""Sharding across GPUs (one process per GPU, torch.distributed).

Kriging targets are independent: every rank holds the whole data set (a
replica of the predictor), predicts one contiguous shard of the targets and
the shards are gathered in rank order -- no collective on the data path
beyond the final gather.  Vecchia log-likelihoods shard by points: each rank
sums the terms of its points and the per-rank partial sums are added in rank
order on the host, so the result does not depend on timing.

The functions take the computation as a callable so that the same host logic
serves the GPU predictors and, in tests, any other implementation.
"""
from __future__ import annotations

from typing import Callable, List, Sequence, Tuple

import numpy as np


def shard_range(n: int, rank: int, world: int) -> Tuple[int, int]:
    """Contiguous [lo, hi) share of n items for `rank` of `world`; the first
    n % world ranks take one extra item."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside world of {world}")
    base, extra = divmod(int(n), int(world))
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def _dist():
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized():
        raise RuntimeError("torch.distributed is not initialised")
    return dist


def predict_sharded(predict: Callable[[np.ndarray], Sequence[np.ndarray]],
                    targets: np.ndarray) -> List[np.ndarray]:
    """Each rank predicts its shard of `targets` with `predict` (returning a
    tuple of per-target arrays, e.g. (value, variance)); every rank receives
    the full arrays, shards concatenated in rank order."""
    dist = _dist()
    rank, world = dist.get_rank(), dist.get_world_size()
    lo, hi = shard_range(len(targets), rank, world)
    mine = [np.asarray(a) for a in predict(targets[lo:hi])]
    parts: List = [None] * world
    dist.all_gather_object(parts, mine)
    return [np.concatenate([p[i] for p in parts]) for i in range(len(mine))]


def sum_sharded(partial: Callable[[int, int], np.ndarray], n: int) -> np.ndarray:
    """Each rank evaluates `partial(lo, hi)` -- per-candidate sums over its
    items [lo, hi) -- and every rank receives the sum of the partials taken in
    rank order (a fixed order, independent of which rank finishes first)."""
    dist = _dist()
    rank, world = dist.get_rank(), dist.get_world_size()
    lo, hi = shard_range(n, rank, world)
    mine = np.asarray(partial(lo, hi), dtype=np.float64)
    parts: List = [None] * world
    dist.all_gather_object(parts, mine)
    total = np.zeros_like(mine)
    for p in parts:
        total = total + p
    return total
