"""Replica bookkeeping for runs on several GPUs.

Scenarios are independent (their own Jacobians, factors and Newton
iterations), so N GPUs run N replicas: every rank solves its own shard of the
scenarios with its own handles, no data crosses between ranks on the hot path,
and only the timing (max over ranks) and, when wanted, the per-scenario results
(gathered to rank 0 on the host) are exchanged.
"""
from __future__ import annotations

import numpy as np


def shard(total: int, rank: int, world: int) -> range:
    """Scenario indices of `rank`: contiguous blocks, sizes differing by at most one."""
    base, extra = divmod(total, world)
    start = rank * base + min(rank, extra)
    return range(start, start + base + (1 if rank < extra else 0))


def max_over_ranks(value: float, dist=None, device=None) -> float:
    """The slowest rank's value (the job's time); `value` itself without dist."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    import torch

    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def gather_columns(local: np.ndarray, dist=None) -> np.ndarray | None:
    """Concatenates the ranks' per-scenario columns ([rows, local scenarios])
    in rank order on rank 0 (None elsewhere); host memory only."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return local
    parts = [None] * dist.get_world_size()
    dist.all_gather_object(parts, np.ascontiguousarray(local))
    return np.concatenate(parts, axis=1) if dist.get_rank() == 0 else None
