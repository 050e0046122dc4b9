"""Replica bookkeeping of multi-GPU runs (one independent frame per rank, no collective on the
data path). The path does not shard a frame across GPUs: each rank renders its own seeded
frame, and the whole-job throughput is the sum of the ranks' units over the slowest rank's time.
"""
from __future__ import annotations


def rank_seed(base_seed: int, rank: int) -> int:
    """Seed of rank `rank`'s frame: ranks render different frames of the same workload."""
    return int(base_seed) + int(rank)


def aggregate(local_ms: float, local_units: float, dist=None, device=None):
    """(units per second over all ranks, max time over ranks in ms, total units).

    `dist` is torch.distributed when a process group is up (None for one process); `device`
    is where the reduction tensors live (a CUDA device for NCCL, None / cpu for gloo)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return local_units / (local_ms / 1e3), float(local_ms), float(local_units)
    import torch
    t = torch.tensor([float(local_ms)], dtype=torch.float64, device=device)
    u = torch.tensor([float(local_units)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    max_ms, units = float(t.item()), float(u.item())
    return units / (max_ms / 1e3), max_ms, units
