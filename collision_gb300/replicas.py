"""Running independent replicas on several GPUs, one process per GPU.

A scene does not shard (every detection pass needs all of its contacts
before velocities update, and impact zones are global union-find
components), so several GPUs run replicas: each rank resolves its own
batch of scenes - its own seed of a workload, or its share of one list of
scenes - with no collective on the data path. The only collectives are
the ones timing needs: a barrier around the timed region and the maximum
of the ranks' times.
"""
from __future__ import annotations

import os


def dist_env():
    """(world size, rank, local rank) from the torchrun environment."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def rank_seed(seed: int, rank: int) -> int:
    """Seed of rank `rank`'s replica of a seeded workload."""
    return seed + rank


def shard(items, rank: int, world: int):
    """Rank `rank`'s share of a list of independent scenes: a contiguous
    run, sizes differing by at most one."""
    n = len(items)
    lo = (n * rank) // world
    hi = (n * (rank + 1)) // world
    return items[lo:hi]


def max_over_ranks(value: float, device=None) -> float:
    """The largest value over all ranks (the job's time is its slowest
    rank's); the value itself when not distributed."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(value: float, device=None) -> float:
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())
