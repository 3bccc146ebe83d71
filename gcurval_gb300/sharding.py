"""One batch split over the ranks of a job, one GPU per rank.

Curves are independent: no knot interval or sample crosses curves and every
prefix sum is per curve, so a batch splits into contiguous ranges of curves
with no exchange during the work; only the results are gathered (an
all-gather of each rank's lengths and sample parameters, in curve order).
The ranges balance the work estimate of ``datasets.cost_proxy`` (knot
intervals weighted by their tens of integrand evaluations, plus samples):
rank r takes the curves whose cumulative cost falls in [r, r + 1) / world of
the total.

    ranges = shard_ranges(batch, world)
    L, u = sharded_run(batch, compute, dist)    # compute(sub) -> (L, u) of a sub-batch

``compute`` runs on the rank's own device (``ArclengthCalculateGpu``), or on
the host (the CPU tests use the oracle).  A curve's result depends only on
that curve, up to the order of the double-double sums of its cumulative
table, which the GPU scan takes in tiles of intervals: a sharded GPU run
agrees with an unsharded one to those sums' rounding.
"""
from __future__ import annotations

import numpy as np

from . import datasets as ds


def shard_ranges(batch: "ds.CurveBatch", world: int) -> list[tuple[int, int]]:
    """Contiguous curve ranges [lo, hi) for ranks 0 .. world - 1, balanced by
    cumulative cost; every range is non-empty while there are at least as
    many curves as ranks."""
    if world < 1:
        raise ValueError("world must be >= 1")
    n = batch.n_curve
    if n == 0:
        return [(0, 0)] * world
    cost = np.cumsum(ds.cost_proxy(batch))
    total = cost[-1]
    cuts = [0]
    for r in range(1, world):
        c = int(np.searchsorted(cost, total * r / world, side="left")) + 1
        # at least one curve per rank (while curves last), non-decreasing
        c = max(c, cuts[-1] + (1 if cuts[-1] < n else 0))
        c = min(c, n - (world - r) if n >= world else n)
        cuts.append(max(c, cuts[-1]))
    cuts.append(n)
    return [(cuts[r], cuts[r + 1]) for r in range(world)]


def shard(batch: "ds.CurveBatch", rank: int, world: int):
    """(lo, hi, sub-batch) of this rank, positions included."""
    lo, hi = shard_ranges(batch, world)[rank]
    sub = batch.subset(np.arange(lo, hi))
    if batch.positions is not None:
        so = np.concatenate([[0], np.cumsum(batch.n_samples.astype(np.int64))])
        sub.positions = batch.positions[so[lo]:so[hi]].copy()
    return lo, hi, sub


def _all_gather_var(x: np.ndarray, dist) -> list[np.ndarray]:
    """All ranks' 1-D float64 arrays of varying length, in rank order."""
    import torch
    t = torch.from_numpy(np.ascontiguousarray(x, np.float64))
    n = torch.tensor([t.numel()], dtype=torch.int64)
    world = dist.get_world_size()
    sizes = [torch.zeros(1, dtype=torch.int64) for _ in range(world)]
    dist.all_gather(sizes, n)
    m = int(max(int(s.item()) for s in sizes))
    buf = torch.zeros(max(m, 1), dtype=torch.float64)
    buf[:t.numel()] = t
    parts = [torch.zeros(max(m, 1), dtype=torch.float64) for _ in range(world)]
    dist.all_gather(parts, buf)
    return [p[:int(s.item())].numpy().copy() for p, s in zip(parts, sizes)]


def sharded_run(batch: "ds.CurveBatch", compute, dist=None):
    """Lengths and sample parameters of the whole batch, each rank computing
    its own contiguous share with ``compute(sub) -> (lengths, us)`` and the
    results gathered to every rank (in curve order).  Without a process
    group, one rank computes everything."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return compute(batch)
    rank, world = dist.get_rank(), dist.get_world_size()
    _, _, sub = shard(batch, rank, world)
    L, u = compute(sub)
    Ls = _all_gather_var(np.asarray(L, np.float64), dist)
    us = _all_gather_var(np.asarray(u, np.float64), dist)
    return np.concatenate(Ls), np.concatenate(us)
