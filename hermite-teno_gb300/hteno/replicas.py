"""Replica bookkeeping for runs on several GPUs: the path has no exchange step, so every rank
advances its own independent grids; a measured quantity is reduced over ranks on the host side
(times: the slowest rank; work: the sum).  Works with the NCCL backend on GPUs and with gloo on
CPU (the multi-process tests)."""
from __future__ import annotations


def world_info():
    import os

    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def reduce(torch, value: float, op: str = "max", device: str = "cpu") -> float:
    """All-reduce of one float over the default process group (identity without one)."""
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op={"max": dist.ReduceOp.MAX, "sum": dist.ReduceOp.SUM, "min": dist.ReduceOp.MIN}[op])
    return float(t.item())


def aggregate_rate(torch, units: float, seconds: float, device: str = "cpu") -> float:
    """Whole-job rate of weak-scaled replicas: all ranks' units over the slowest rank's time."""
    return reduce(torch, units, "sum", device) / reduce(torch, seconds, "max", device)
