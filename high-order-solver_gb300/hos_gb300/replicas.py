"""Runs on several GPUs of one node: independent replicas, one process per GPU.

A step of one problem does not shard here (the path fixes one GPU per problem), so N GPUs run
N independent copies of the workload: no data crosses between ranks.  The ranks meet only to
time the run: a barrier before the timed region, and the slowest rank's time (max over ranks)
for the whole-job throughput, N x the units one rank processed / that time.

The rank layout comes from the launcher's environment (torchrun: WORLD_SIZE, RANK,
LOCAL_RANK, MASTER_ADDR, MASTER_PORT).  The process group is NCCL on GPUs; the same calls run
over gloo on the CPU in the tests.
"""
from __future__ import annotations

import os


def env() -> tuple[int, int, int]:
    """(world size, rank, local rank) from the launcher's environment; (1, 0, 0) alone."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def barrier(world_size: int) -> None:
    """All ranks reach this point before any continues (no-op for one rank)."""
    if world_size > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(value: float, world_size: int, device=None) -> float:
    """The largest of the ranks' values (the slowest rank's time); device: where the
    collective's buffer lives (a CUDA device for NCCL, None for gloo on the CPU)."""
    if world_size <= 1:
        return float(value)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_rate(world_size: int, units_per_rank: float, seconds_max: float) -> float:
    """Whole-job throughput of independent replicas: every rank processed units_per_rank, the
    job took the slowest rank's time."""
    return world_size * units_per_rank / seconds_max
