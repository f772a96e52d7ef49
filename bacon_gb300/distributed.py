"""Multi-GPU use of the engine: independent shards, no data exchange.

Systems are independent, so a batch splits into contiguous shards, one per
rank (one process per GPU).  The only collectives are the ones a benchmark or
a caller needs around the solve: a barrier, the maximum of the per-rank times,
and optionally gathering the per-system results.
"""
from __future__ import annotations

import numpy as np

from .workloads import Batch


def shard_range(n: int, rank: int, world: int) -> tuple[int, int]:
    """[start, stop) of rank's contiguous shard; sizes differ by at most one."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank / world size")
    base, extra = divmod(n, world)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def shard(batch: Batch, rank: int, world: int) -> Batch:
    start, stop = shard_range(batch.n, rank, world)
    return batch.subset(np.arange(start, stop))


def max_over_ranks(value: float, dist, device=None) -> float:
    """Maximum of a per-rank scalar (the time of the slowest rank)."""
    import torch
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def gather_columns(local: np.ndarray, n_total: int, dist) -> np.ndarray:
    """Concatenate per-rank (..., n_local) arrays along the last axis, in rank
    order (the inverse of shard)."""
    import torch
    world = dist.get_world_size()
    parts = [None] * world
    dist.all_gather_object(parts, np.ascontiguousarray(local))
    out = np.concatenate(parts, axis=-1)
    if out.shape[-1] != n_total:
        raise RuntimeError("gathered shards do not cover the batch")
    return out
