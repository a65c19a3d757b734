"""Replica runs: one independent structure function per rank, no data exchange.

Image stacks are independent and one stack fits one GB300, so N GPUs run N
replicas of the computation (one process per GPU, launched by
``torch.distributed.run``).  The only collectives are a barrier on each side
of a timed region and the maximum of the ranks' times, over whichever backend
the process group uses (NCCL between GPUs, gloo in the CPU tests).
"""

from __future__ import annotations

import os


def world() -> tuple[int, int, int]:
    """(world size, rank, local rank) from the launcher's environment; (1, 0, 0) when run alone."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def _group_active() -> bool:
    import torch.distributed as dist

    return dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1


def barrier() -> None:
    """Wait for every rank (no-op without a process group of more than one rank)."""
    if _group_active():
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(value: float, device=None) -> float:
    """The largest `value` over all ranks (the job's time is its slowest replica's)."""
    if not _group_active():
        return float(value)
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_rate(units_per_rank: float, seconds: float, world_size: int) -> float:
    """Whole-job throughput: the units all replicas processed over the slowest replica's time."""
    if seconds <= 0:
        raise ValueError("seconds must be positive")
    return world_size * units_per_rank / seconds
