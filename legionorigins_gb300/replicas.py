"""Replica runs across processes (one per GPU).

The circuit path has no exchange between independent circuits, so several
GPUs run replicas: every rank simulates its own circuit, and the job's rate
is all ranks' work over the slowest rank's time.  This module holds that
aggregation so it can be exercised with the gloo backend on CPU.
"""
from __future__ import annotations


def aggregate(local_updates: float, local_seconds: float, device: str = "cpu"):
    """Returns (total updates over all ranks, max seconds over ranks, world
    size).  Without an initialised process group it is the local values."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()):
        return float(local_updates), float(local_seconds), 1
    u = torch.tensor([float(local_updates)], dtype=torch.float64, device=device)
    t = torch.tensor([float(local_seconds)], dtype=torch.float64, device=device)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(u.item()), float(t.item()), dist.get_world_size()


def rate(local_updates: float, local_seconds: float, device: str = "cpu") -> float:
    """Whole-job wire-segment updates per second."""
    total, seconds, _ = aggregate(local_updates, local_seconds, device)
    return total / seconds if seconds > 0 else 0.0
