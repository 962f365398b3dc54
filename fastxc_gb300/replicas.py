"""Host logic of multi-GPU runs. The correlation path shards without a
data-path collective: timestamps (days), pair blocks, station-days and stack
pairs are independent (fastxc/distributed/planner.py:169-186,
native/xc/worker/scheduler.cu:43-63). One process drives one GPU; the only
reduction is the cross-day linear stack, a weighted sum of per-shard stacks
done once on the host side (or as one all-reduce of npairs x nspec values).
"""

from __future__ import annotations

import numpy as np


def dist_env() -> tuple[int, int, int]:
    """(rank, world, local_rank) from the torchrun environment."""
    import os

    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def day_shard(ndays: int, rank: int, world: int) -> range:
    """Contiguous share of [0, ndays) for `rank`: sizes differ by at most one
    day and the shards cover every day exactly once."""
    lo = ndays * rank // world
    hi = ndays * (rank + 1) // world
    return range(lo, hi)


def reduce_max(value: float, device=None) -> float:
    """Maximum of a scalar over all ranks (the timed region of a replica
    run is the slowest rank's)."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def linear_stack_over_shards(stack: np.ndarray, windows: int) -> tuple[np.ndarray, int]:
    """Cross-shard linear stack: every rank holds the mean over its own
    `windows` windows; the result is the mean over all windows of all ranks
    (sum of stack x windows, divided by the total), the same as one rank
    stacking every window. Returns (mean stack, total windows)."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return stack, windows
    s = torch.from_numpy(np.ascontiguousarray(stack, np.complex128).view(np.float64).copy())
    w = torch.tensor([float(windows)], dtype=torch.float64)
    s *= float(windows)
    dist.all_reduce(s)
    dist.all_reduce(w)
    total = int(round(w.item()))
    out = (s / max(total, 1)).numpy().view(np.complex128).reshape(stack.shape)
    return out, total


def whole_job_rate(units_per_rank: float, world: int, seconds_max: float) -> float:
    """Aggregate throughput of a weak-scaling replica run: the units all
    ranks processed over the slowest rank's time."""
    return units_per_rank * world / seconds_max if seconds_max > 0 else 0.0
