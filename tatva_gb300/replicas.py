"""Replicas across GPUs: one process per GPU, each running the same workload on its
own device with no data-path collective (the hot path here does not shard).  Only
the timing is combined: a barrier before and after the timed region, the slowest
rank's time, and the sum of the units all ranks processed.

Launch with ``torchrun --nproc-per-node N`` (RANK / LOCAL_RANK / WORLD_SIZE /
MASTER_ADDR / MASTER_PORT from the environment); NCCL on GPUs, gloo on CPU.
"""

from __future__ import annotations

import os

import torch
import torch.distributed as dist


def world() -> tuple[int, int, int]:
    """(world_size, rank, local_rank) from the launcher's environment."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def init(backend: str | None = None) -> None:
    ws, _, _ = world()
    if ws > 1 and not dist.is_initialized():
        dist.init_process_group(backend or ("nccl" if torch.cuda.is_available() else "gloo"))


def _device():
    if dist.get_backend() == "nccl":
        return torch.device("cuda", torch.cuda.current_device())
    return torch.device("cpu")


def barrier() -> None:
    if dist.is_initialized():
        dist.barrier()


def max_over_ranks(x: float) -> float:
    """The slowest rank's value (timings)."""
    if not dist.is_initialized():
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=_device())
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(x: float) -> float:
    """Units processed by all ranks together."""
    if not dist.is_initialized():
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=_device())
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def aggregate_throughput(units_per_rank: float, seconds_per_rank: float) -> float:
    """Whole-job throughput of weak-scaled replicas: all ranks' units over the slowest
    rank's time."""
    return sum_over_ranks(units_per_rank) / max_over_ranks(seconds_per_rank)


__all__ = ["aggregate_throughput", "barrier", "init", "max_over_ranks", "sum_over_ranks", "world"]
