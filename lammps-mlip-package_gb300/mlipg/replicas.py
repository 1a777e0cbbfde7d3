"""Replica bookkeeping for multi-GPU runs of independent copies of a workload.

The path does not exchange data between GPUs: each rank evaluates its own
replica and only the timing is combined (barrier before and after the timed
region, maximum of the ranks' times).  Works with any torch.distributed
backend; the host-side logic is tested with gloo on CPU.
"""
from __future__ import annotations

import os


def world():
    """(rank, world size) from the launcher's environment."""
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1"))


def init(backend: str = "gloo") -> dict:
    rank, size = world()
    if size > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        if not dist.is_initialized():
            dist.init_process_group(backend)
    return {"rank": rank, "world": size}


def barrier(info: dict) -> None:
    if info["world"] > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(value: float, info: dict) -> float:
    """The largest of the ranks' values (the slowest replica sets the time)."""
    if info["world"] <= 1:
        return float(value)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_rate(units_per_rank: float, seconds: float, info: dict) -> float:
    """Whole-job throughput of weak-scaled replicas: all ranks' units over the
    slowest rank's time."""
    return units_per_rank * info["world"] / max_over_ranks(seconds, info)


def finish(info: dict) -> None:
    if info["world"] > 1:
        import torch.distributed as dist
        if dist.is_initialized():
            dist.destroy_process_group()
