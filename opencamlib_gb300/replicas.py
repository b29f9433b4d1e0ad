"""Replica driver: one process per GPU, each running the whole workload on
its own device (CL points and fibers are independent and the mesh is
replicated, so there is no data-path collective).  The process group only
carries the barriers around a timed region and the maximum of the ranks'
times.  Used by bench.py; torchrun (or any launcher that sets RANK,
WORLD_SIZE, LOCAL_RANK, MASTER_ADDR, MASTER_PORT) starts the ranks.
"""
from __future__ import annotations

import os


def setup(backend: str = "nccl"):
    """(rank, world, local_rank, dist or None) from the launcher's
    environment; a single process needs no process group."""
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world <= 1:
        return 0, 1, 0, None
    import torch.distributed as dist
    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    if not dist.is_initialized():
        dist.init_process_group(backend)
    return rank, world, local, dist


def barrier(dist) -> None:
    if dist is not None:
        dist.barrier()


def max_over_ranks(x: float, dist, device: str = "cpu") -> float:
    """The largest x over all ranks (the timed region ends with the slowest
    replica)."""
    if dist is None:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank: float, world: int, seconds: float) -> float:
    """Units per second of the whole job: every rank processed its own
    units, and the job took the slowest rank's time."""
    return world * units_per_rank / seconds


def teardown(dist) -> None:
    if dist is not None and dist.is_initialized():
        dist.destroy_process_group()
