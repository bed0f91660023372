"""Replica bookkeeping for multi-GPU runs of independent problems.

The f(A)b path does not shard at the sizes it targets, so N GPUs run N
independent replicas. One process per GPU, each with its own engine and its
own right-hand sides. There is no collective on the data path. Only the
timing is combined:
- the job's time is the slowest rank's time (a max all-reduce);
- its throughput is all ranks' units over that time.

The functions accept any initialised process group: NCCL on GPUs, or gloo for
the CPU tests.
"""
from __future__ import annotations

from typing import Sequence

__all__ = ["max_over_ranks", "job_throughput", "rank0_only"]


def max_over_ranks(values: Sequence[float], device=None) -> list:
    """Element-wise maximum of ``values`` over all ranks (identity without a group)."""
    import torch
    import torch.distributed as dist
    vals = [float(v) for v in values]
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return vals
    t = torch.tensor(vals, dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t.tolist()]


def job_throughput(units_per_rank: float, ms_per_step_local: float, world: int, device=None):
    """(units/s of the whole job, slowest rank's ms per step).

    Every rank processes ``units_per_rank`` per step, so the job processes
    world * units_per_rank per step in the slowest rank's time."""
    (ms,) = max_over_ranks([ms_per_step_local], device=device)
    return world * units_per_rank * 1e3 / ms, ms


def rank0_only(rank: int) -> bool:
    """The reference arm runs on rank 0 only; the other ranks exit without work."""
    return rank == 0
