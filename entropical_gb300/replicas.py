"""Multi-GPU: independent shards, one process per GPU.

The density path splits into independent objects (densities, hence MI pairs,
TE (pair, lag) entries, trajectories), so N GPUs never exchange data on the
path. Two forms:

* weak scaling (bench.py under torchrun): every rank computes its own
  problem of the benchmark's size (rank r: the benchmark data with seed +r);
  the report takes the sum of the work and the maximum of the step times
  over ranks (``aggregate``);
* one problem split over ranks (``mi_all_pairs_sharded``): the 64 + 2016
  densities of an all-pairs MI are dealt out in contiguous shares, every
  rank computes the entropies of its share as one batch, and the small vector
  of entropies is gathered on the host to assemble the MI matrix.

Only the report and the final scalars cross ranks; no collective is on the
data path.
"""
from __future__ import annotations

from typing import Callable, Sequence

import numpy as np


def aggregate(units: float, ms: float, dist=None, device=None) -> tuple[float, float]:
    """(sum of units over ranks, max of ms over ranks); identity without dist."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(units), float(ms)
    import torch
    t = torch.tensor([float(units), float(ms)], dtype=torch.float64,
                     device=device if device is not None else "cpu")
    u = t[:1].clone()
    m = t[1:].clone()
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    dist.all_reduce(m, op=dist.ReduceOp.MAX)
    return float(u.item()), float(m.item())


def shard(n_items: int, rank: int, world: int) -> range:
    """Contiguous share of n_items for one rank."""
    base, extra = divmod(n_items, world)
    start = rank * base + min(rank, extra)
    return range(start, start + base + (1 if rank < extra else 0))


def mi_instances(n_cols: int) -> list[tuple[int, ...]]:
    """The densities of an all-pairs MI in batch order: (i,) for the 1-D
    marginals, then (i, j) for i < j."""
    return [(i,) for i in range(n_cols)] + [(i, j) for i in range(n_cols)
                                            for j in range(i + 1, n_cols)]


def mi_all_pairs_sharded(entropies: Callable[[list], np.ndarray], x: np.ndarray,
                         h: Sequence[float], dist=None) -> tuple[np.ndarray, np.ndarray]:
    """All-pairs resubstitution MI of the rows of x (n_cols, n_rows) with the
    densities split over the ranks of dist. ``entropies`` maps a list of
    [(coords (d, n), h (d,))...] to their entropies as one batch (e.g.
    Context.entropy_batch on this rank's GPU). Returns (MI, marginal
    entropies), the same on every rank."""
    M = x.shape[0]
    inst = mi_instances(M)
    world = dist.get_world_size() if dist is not None and dist.is_initialized() else 1
    rank = dist.get_rank() if world > 1 else 0
    mine = shard(len(inst), rank, world)
    batch = [(np.ascontiguousarray(x[list(c)]), np.asarray([h[k] for k in c], np.float32))
             for c in (inst[q] for q in mine)]
    H_mine = np.asarray(entropies(batch), np.float64) if batch else np.zeros(0)
    if world > 1:
        parts = [None] * world
        dist.all_gather_object(parts, (mine.start, H_mine.tolist()))
        H = np.zeros(len(inst))
        for start, vals in parts:
            H[start:start + len(vals)] = vals
    else:
        H = H_mine
    mi = np.zeros((M, M))
    for q, c in enumerate(inst):
        if len(c) == 2:
            i, j = c
            mi[i, j] = mi[j, i] = H[i] + H[j] - H[q]
    return mi, H[:M].copy()
