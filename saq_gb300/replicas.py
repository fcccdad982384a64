"""Replica timing for runs on several GPUs.

The search has no exchange step between GPUs: `bench.py --gpus N` runs N
independent replicas, one process per GPU, each answering its own batches.
Whole-job throughput is every rank's units over the slowest rank's time, so
each rank contributes its elapsed time to a max-reduction.
"""
from __future__ import annotations


def max_over_ranks(x: float, device: str = "cuda") -> float:
    """The largest `x` over all ranks (itself when not distributed).  `device`
    is where the reduction tensor lives: "cuda" for NCCL, "cpu" for gloo."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(units_per_rank: int, my_seconds: float, world: int, device: str = "cuda") -> float:
    """Units per second of the whole job: world x units_per_rank over the
    slowest rank's seconds."""
    return world * units_per_rank / max_over_ranks(my_seconds, device)
