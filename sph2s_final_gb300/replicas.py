"""Host-side coordination for one process per GPU on one node.

A single scene's step is one global neighbour computation with no exchange-free
partition, so several GPUs run independent replicas of the workload (weak
scaling, no collective on the data path).  Independent scenes (a batch) are
sharded whole across ranks.  The only collectives are the timing barrier and
the max over ranks of the timed region, taken on a process group that may be
NCCL (GPU runs) or gloo (the CPU tests).
"""
from __future__ import annotations

import os


def world() -> tuple[int, int, int]:
    """(world size, rank, local rank) from the torchrun environment (1, 0, 0 if absent)."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def shard(num_units: int, rank: int, world_size: int) -> range:
    """Contiguous, balanced share of `num_units` independent units (scenes) for
    `rank`; the shares of all ranks are disjoint and cover every unit."""
    if world_size < 1 or not 0 <= rank < world_size:
        raise ValueError(f"bad rank {rank} of {world_size}")
    base, extra = divmod(num_units, world_size)
    start = rank * base + min(rank, extra)
    return range(start, start + base + (1 if rank < extra else 0))


def _dist():
    import torch.distributed as dist
    return dist if dist.is_available() and dist.is_initialized() else None


def barrier() -> None:
    d = _dist()
    if d is not None:
        d.barrier()


def max_over_ranks(value: float, device=None) -> float:
    """The maximum of `value` over all ranks (the identity without a process group)."""
    d = _dist()
    if d is None:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    d.all_reduce(t, op=d.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(value: float, device=None) -> float:
    d = _dist()
    if d is None:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    d.all_reduce(t, op=d.ReduceOp.SUM)
    return float(t.item())


def throughput(units_all_ranks: float, ms_max: float) -> float:
    """Whole-job units per second: everything all ranks processed over the
    slowest rank's timed region."""
    return units_all_ranks / (ms_max * 1e-3)
