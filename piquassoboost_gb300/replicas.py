"""Replica aggregation for multi-GPU runs.

The permanent path runs one independent replica per GPU (no collective on
the data path).  The only cross-rank step is the bench's aggregate: total
units over all ranks divided by the slowest rank's time.
"""
from __future__ import annotations


def replica_throughput(local_units: float, local_seconds: float, device=None) -> tuple[float, float]:
    """(sum of units over ranks / max seconds over ranks, max seconds).

    Works with any initialised torch.distributed backend (NCCL with a CUDA
    device, gloo on CPU); without a process group it is the local ratio."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return local_units / local_seconds, local_seconds
    dev = device if device is not None else "cpu"
    t = torch.tensor([float(local_seconds)], dtype=torch.float64, device=dev)
    u = torch.tensor([float(local_units)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return u.item() / t.item(), t.item()


def shard_seeds(base_seed: int, rank: int, steps: int) -> list[int]:
    """Per-rank seeds of a replica's workload (disjoint across ranks)."""
    return [base_seed + 1000 * rank + s for s in range(steps)]
