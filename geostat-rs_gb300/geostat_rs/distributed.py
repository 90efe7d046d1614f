"""Sharding across GPUs (one process per GPU, torch.distributed).

Kriging targets are independent: every rank holds the whole data set (a
replica of the predictor), predicts one contiguous shard of the targets and
the shards are gathered in rank order -- no collective on the data path
beyond the final gather.  Vecchia log-likelihoods shard by points: each rank
sums the terms of its ordered positions (``VecchiaPlan.loglik_range``) and
the per-rank partial sums are added in rank order on the host, so the result
does not depend on timing.

Results travel as arrays (``all_gather`` of tensors padded to the largest
shard), never as pickled objects.  The functions take the computation as a
callable so that the same host logic serves the GPU predictors and, in
tests, any other implementation.
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


def _gather_rows(dist, mine: np.ndarray, counts: Sequence[int]) -> np.ndarray:
    """All ranks' 1-D arrays (rank r holds counts[r] items) concatenated in
    rank order, exchanged as host tensors padded to the largest count."""
    import torch
    width = max(max(counts), 1)
    buf = np.zeros(width, dtype=mine.dtype)
    buf[:len(mine)] = mine
    t = torch.from_numpy(buf)
    parts = [torch.empty_like(t) for _ in counts]
    dist.all_gather(parts, t)
    return np.concatenate([p.numpy()[:c] for p, c in zip(parts, counts)])


def predict_sharded(predict: Callable[[np.ndarray], Sequence[np.ndarray]],
                    targets: np.ndarray) -> List[np.ndarray]:
    """Each rank predicts its shard of `targets` with `predict` (returning a
    tuple of per-target 1-D arrays, e.g. (value, variance, status)); every
    rank receives the full arrays, shards concatenated in rank order."""
    dist = _dist()
    rank, world = dist.get_rank(), dist.get_world_size()
    n = len(targets)
    lo, hi = shard_range(n, rank, world)
    mine = [np.ascontiguousarray(a).reshape(-1) for a in predict(targets[lo:hi])]
    counts = [b - a for a, b in (shard_range(n, r, world) for r in range(world))]
    return [_gather_rows(dist, a, counts) for a in mine]


def sum_sharded(partial: Callable[[int, int], np.ndarray], n: int) -> np.ndarray:
    """Each rank evaluates `partial(lo, hi)` -- per-candidate sums over its
    items [lo, hi) -- and every rank receives the sum of the partials taken in
    rank order (a fixed order, independent of which rank finishes first)."""
    import torch
    dist = _dist()
    rank, world = dist.get_rank(), dist.get_world_size()
    lo, hi = shard_range(n, rank, world)
    mine = np.ascontiguousarray(partial(lo, hi), dtype=np.float64).reshape(-1)
    t = torch.from_numpy(mine.copy())
    parts = [torch.empty_like(t) for _ in range(world)]
    dist.all_gather(parts, t)
    total = np.zeros_like(mine)
    for p in parts:
        total = total + p.numpy()
    return total
