"""Multi-GPU: independent shards, one process per GPU.

The density path splits into independent objects (densities, hence MI pairs,
TE (pair, lag) entries, trajectories), so N GPUs never exchange data on the
path. Three forms:

* weak scaling (bench.py under torchrun): every rank computes its own
  problem of the benchmark's size (rank r: the benchmark data with seed +r);
  the report takes the sum of the work and the maximum of the step times
  over ranks (``aggregate``);
* one job split over ranks (``mi_all_pairs_split``, ``te_all_pairs_split``):
  every rank holds the coordinate matrix in its own device memory (one
  upload), computes the entropies of its share of the job's densities as one
  batch (``Context.mi_entropies_device`` / ``te_entropies_device``: only the
  views its share uses are sorted), and the entropies -- a few KB -- are
  gathered on the host to assemble the MI matrix or the TE tensor. Shares are
  dealt by an estimate of each density's cost (``WEIGHTS``), not by count;
* one density split over ranks (``densities_split``), as the reference's
  per-GPU driver splits its target rows (density_1d.cuh:181-219): every rank
  computes one share of the targets against every source
  (``Context.combined_densities_part_device``) into a zeroed buffer, and the
  shares are added on the host (each target is written by one rank only).

Only the report, the final scalars or the per-point densities of a split
density cross ranks; no collective is on the data path.
"""
from __future__ import annotations

from typing import Callable, Sequence

import numpy as np

# Relative cost of one density by dimension, from the measured per-dimension
# kernel times of the benchmark batches on one GB300 (all-pairs MI 64 x 100k:
# 64 1-D in 0.26 ms, 2,016 2-D in ~50 ms; TE 32 x 200k x 3 lags: 1,584 2-D in
# ~210 ms, 2,976 3-D in ~770 ms), per point.
WEIGHTS = {1: 0.005, 2: 1.0, 3: 2.0}


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


def deal(weights: Sequence[float], world: int) -> list[np.ndarray]:
    """Shares of items with the given costs: the heaviest item goes to the
    least loaded rank, in turn (ties: the lower rank, the lower index).
    Returns one sorted index array per rank; together they hold every item
    once."""
    w = np.asarray(weights, dtype=np.float64)
    order = np.argsort(-w, kind="stable")
    load = np.zeros(world)
    owner = np.empty(len(w), dtype=np.int64)
    for i in order:
        r = int(np.argmin(load))
        owner[i] = r
        load[r] += w[i]
    return [np.flatnonzero(owner == r).astype(np.uint64) for r in range(world)]


def mi_instances(n_cols: int) -> list[tuple[int, ...]]:
    """The densities of an all-pairs MI in batch order: (i,) for the 1-D
    marginals, then (i, j) for i < j."""
    return [(i,) for i in range(n_cols)] + [(i, j) for i in range(n_cols)
                                            for j in range(i + 1, n_cols)]


def te_instances(n_cols: int, n_taus: int) -> list[tuple[int, int, int, int]]:
    """The densities of an all-ordered-pairs TE in batch order, as (lag index,
    kind, i, j): kind 1 the 1-D y_i, 2 the lagged (y_i+, y_i), 3 the joint
    (y_i, x_j) for i < j, 4 the 3-D (y_i+, y_i, x_j) for i != j."""
    M = n_cols
    out = []
    for q in range(n_taus):
        out += [(q, 1, i, i) for i in range(M)]
        out += [(q, 2, i, i) for i in range(M)]
        out += [(q, 3, i, j) for i in range(M) for j in range(i + 1, M)]
        out += [(q, 4, i, j) for i in range(M) for j in range(M) if i != j]
    return out


def _world(dist) -> tuple[int, int]:
    if dist is not None and dist.is_initialized() and dist.get_world_size() > 1:
        return dist.get_rank(), dist.get_world_size()
    return 0, 1


def split_entropies(entropies_of: Callable[[np.ndarray], np.ndarray],
                    weights: Sequence[float], dist=None) -> np.ndarray:
    """Entropies of every item of a job, each rank computing its dealt share
    with ``entropies_of(item indices)``; gathered on the host of every rank."""
    rank, world = _world(dist)
    shares = deal(weights, world)
    mine = shares[rank]
    H_mine = np.asarray(entropies_of(mine), np.float64) if len(mine) else np.zeros(0)
    if world == 1:
        return H_mine
    parts = [None] * world
    dist.all_gather_object(parts, (rank, H_mine.tolist()))
    H = np.zeros(len(weights))
    for r, vals in parts:
        H[shares[r]] = vals
    return H


def mi_assemble(n_cols: int, H: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """MI matrix and marginal entropies from the entropies in MI batch order."""
    M = n_cols
    mi = np.zeros((M, M))
    k = M
    for i in range(M):
        for j in range(i + 1, M):
            mi[i, j] = mi[j, i] = H[i] + H[j] - H[k]
            k += 1
    return mi, np.asarray(H[:M], np.float64).copy()


def te_assemble(n_cols: int, n_taus: int, H: np.ndarray) -> np.ndarray:
    """TE tensor [lag, i, j] = TE_{j->i} from the entropies in TE batch order."""
    M = n_cols
    per = 2 * M + M * (M - 1) // 2 + M * (M - 1)
    pair = {}
    k = 0
    for i in range(M):
        for j in range(i + 1, M):
            pair[(i, j)] = pair[(j, i)] = k
            k += 1
    te = np.zeros((n_taus, M, M))
    for q in range(n_taus):
        b = q * per
        b2l, b2j, b3 = b + M, b + 2 * M, b + 2 * M + M * (M - 1) // 2
        k3 = 0
        for i in range(M):
            for j in range(M):
                if i == j:
                    continue
                te[q, i, j] = H[b2j + pair[(i, j)]] + H[b2l + i] - H[b3 + k3] - H[b + i]
                k3 += 1
    return te


def mi_all_pairs_split(ctx, d_coords: int, n_rows: int, n_cols: int, h: Sequence[float],
                       dist=None) -> tuple[np.ndarray, np.ndarray]:
    """All-pairs MI of the device matrix d_coords (column-major n_rows x
    n_cols, in this rank's device memory) with the densities dealt over the
    ranks of dist. Returns (MI, marginal entropies), the same on every rank."""
    inst = mi_instances(n_cols)
    w = [WEIGHTS[len(c)] for c in inst]
    H = split_entropies(lambda items: ctx.mi_entropies_device(d_coords, n_rows, n_cols, h, items),
                        w, dist)
    return mi_assemble(n_cols, H)


def te_all_pairs_split(ctx, d_coords: int, n_rows: int, n_cols: int, h: Sequence[float],
                       taus: Sequence[int], dist=None) -> np.ndarray:
    """All-ordered-pairs TE of the device matrix d_coords with the densities
    dealt over the ranks of dist; the same tensor on every rank."""
    inst = te_instances(n_cols, len(taus))
    dim = {1: 1, 2: 2, 3: 2, 4: 3}
    w = [WEIGHTS[dim[kind]] for _, kind, _, _ in inst]
    H = split_entropies(
        lambda items: ctx.te_entropies_device(d_coords, n_rows, n_cols, h, taus, items), w, dist)
    return te_assemble(n_cols, len(taus), H)


def densities_split(ctx, d_coords: int, n_rows: int, n_cols: int, i_cols: Sequence[int],
                    h: Sequence[float], tau: Sequence[int] | None = None,
                    dist=None, device=None) -> tuple[np.ndarray, float]:
    """One density of the device matrix d_coords with its targets split over
    the ranks of dist: rank r computes share r into a zeroed buffer on
    ``device`` (default: the current CUDA device), the shares are summed on
    the host. Returns (densities by original index, entropy -mean log p), the
    same on every rank."""
    import torch
    rank, world = _world(dist)
    n_sel = n_rows - (max(tau) if tau else 0)
    dev = device if device is not None else torch.cuda.current_device()
    buf = torch.zeros(n_sel, dtype=torch.float64, device=dev)
    _, ls = ctx.combined_densities_part_device(d_coords, n_rows, n_cols, i_cols, h, tau, rank,
                                               world, buf.data_ptr())
    p = buf.cpu().numpy()
    if world > 1:
        parts = [None] * world
        dist.all_gather_object(parts, (p, ls))
        p = np.sum([q for q, _ in parts], axis=0)
        ls = float(sum(v for _, v in parts))
    return p, -ls / n_sel
