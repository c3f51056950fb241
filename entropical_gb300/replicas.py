"""Multi-GPU replicas.

The density path shards into independent instances, and every host here has
one GPU, so N GPUs run N independent replicas of a step (one process per GPU,
launched by torchrun). The only cross-rank step is the report: the step time
is the maximum over ranks and the work is the sum over ranks. No collective is
on the data path.
"""
from __future__ import annotations


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
    """Contiguous share of n_items for one rank (for callers that split a batch
    of independent instances across GPUs)."""
    base, extra = divmod(n_items, world)
    start = rank * base + min(rank, extra)
    return range(start, start + base + (1 if rank < extra else 0))
