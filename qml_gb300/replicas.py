"""Replica bookkeeping for runs with one process per GPU.

The path has no data exchange between GPUs.  Each rank fits its own seeded problem,
and the job's step time is the slowest rank's.  This module holds the small amount
of host logic that needs: per-rank seeds, and the max-over-ranks reduction of a
timing, in any torch.distributed backend (nccl on GPUs, gloo on CPU).
"""
from __future__ import annotations

import os

import torch
import torch.distributed as dist


def rank_info():
    """(world, rank, local_rank) from the torchrun environment (1, 0, 0 without it)."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def replica_seed(base_seed: int, rank: int) -> int:
    """Distinct, reproducible seed for each replica's synthetic problem."""
    return int(base_seed) + 1000003 * int(rank)


def max_over_ranks(value: float, device=None) -> float:
    """The largest value over all ranks (the value itself when not distributed)."""
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    dev = device if device is not None else (
        torch.device("cuda", torch.cuda.current_device())
        if dist.get_backend() == "nccl" else torch.device("cpu"))
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(units_per_rank: float, step_seconds_max: float, world: int) -> float:
    """Whole-job rate: the units all ranks processed over the slowest rank's time."""
    return units_per_rank * world / step_seconds_max
