"""Replica parallelism: one process per GPU, each advancing its own grids, with no exchange on
the data path.  Ranks meet only at a barrier around the timed region and in one reduction of
the elapsed time (the whole job lasts as long as its slowest rank).  Ensemble members are
dealt to ranks by index."""
from __future__ import annotations

import os


def dist_info():
    """(rank, world size, local rank) from the launcher's environment (1 process: 0, 1, 0)."""
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def max_over_ranks(x: float, device=None) -> float:
    """Maximum of x over all ranks of the default process group (x itself without one).
    device: where the reduction tensor lives (a CUDA device for NCCL, CPU for gloo)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device or "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank: float, seconds_max: float, world: int) -> float:
    """Units all ranks processed per second of the slowest rank (weak scaling: every rank
    does the same work)."""
    return units_per_rank * world / seconds_max


def shard(n: int, rank: int, world: int):
    """Indices of the n members that rank owns: every world-th member starting at rank, so
    each rank gets the same mix of sizes when members are listed size by size."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank must be in [0, world)")
    return list(range(rank, n, world))
