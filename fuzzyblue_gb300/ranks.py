"""Replica ranks of a multi-GPU run: one process per GPU, each building its own
atmospheres (atmospheres are independent; no collective on the data path).
These helpers give the launch's rank layout, the barrier around a timed
region, the maximum of a per-rank time over all ranks and the whole-job rate.
They work on any torch.distributed backend: NCCL with one GPU per rank, gloo
on CPU (the multi-rank tests)."""
from __future__ import annotations

import os
from typing import Tuple


def layout() -> Tuple[int, int, int]:
    """(world size, rank, local rank) from the torchrun environment."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def barrier(world: int) -> None:
    if world > 1:
        import torch.distributed as td
        td.barrier()


def max_over_ranks(world: int, value: float) -> float:
    """The largest of every rank's `value` (a time: the slowest rank bounds the job)."""
    if world == 1:
        return value
    import torch
    import torch.distributed as td
    device = "cuda" if td.get_backend() == "nccl" else "cpu"
    t = torch.tensor([value], dtype=torch.float64, device=device)
    td.all_reduce(t, op=td.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(world: int, units_per_rank: int, seconds: float) -> float:
    """Units all ranks processed per second of the slowest rank."""
    return world * units_per_rank / seconds
