"""Replica bookkeeping for multi-GPU runs (one inversion per rank, no data-path collective).

A single cube's transform does not shard without an all-to-all, and cubes are
independent, so N GPUs run N independent inversions.  The only cross-rank
communication is timing: a barrier around the timed region and the maximum
step time over ranks.  Works with any torch.distributed backend (nccl on
GPUs, gloo on CPU).
"""
from __future__ import annotations

import os


def world():
    """(world_size, rank, local_rank) from the torchrun environment."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def barrier(world_size):
    if world_size > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x: float, world_size: int, device=None) -> float:
    if world_size == 1:
        return float(x)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(bins_per_rank: int, ms_per_step_max: float, world_size: int) -> float:
    """Total Mbins/s of all replicas: every rank inverts its own cube per step."""
    return bins_per_rank * world_size / (ms_per_step_max * 1e-3) / 1e6
