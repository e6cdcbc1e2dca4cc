"""Multi-GPU handling for the benchmark: the hot path does not shard across GPUs
without changing results (LU-SGS sweeps follow one global cell order), so N GPUs
run N independent replicas of the same solve.  This module holds the only
cross-rank step: agreeing on the timed region and reducing the per-rank
measurements (max of the times, sum of the work).
"""
from __future__ import annotations

import os


def dist_env() -> tuple[int, int, int]:
    """(rank, world_size, local_rank) from the torchrun environment."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def init(backend: str):
    """Initialise torch.distributed when launched with WORLD_SIZE > 1."""
    import torch.distributed as dist
    rank, world, _ = dist_env()
    if world > 1 and not dist.is_initialized():
        dist.init_process_group(backend=backend, rank=rank, world_size=world)
    return dist if world > 1 else None


def barrier(dist, device=None) -> None:
    if dist is None:
        return
    if device is not None and dist.get_backend() == "nccl":
        dist.barrier(device_ids=[device])
    else:
        dist.barrier()


def reduce_timing(dist, units: float, seconds: float, device: str = "cpu") -> tuple[float, float]:
    """Whole-job (units summed over ranks, seconds = max over ranks)."""
    if dist is None:
        return units, seconds
    import torch
    t = torch.tensor([seconds], dtype=torch.float64, device=device)
    u = torch.tensor([units], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return float(u.item()), float(t.item())
