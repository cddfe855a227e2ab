"""Replicas across GPUs: one process per GPU, no data-path collective.

The per-step path does not shard: a single system stays on one GPU.  What
spreads over GPUs is independent work: bench replicas of the same workload,
the systems of an ensemble, the requests of a served stream.  Each rank
takes its share of the items (`shard`), runs it alone, and the ranks meet
only to report: the slowest rank's time (`max_over_ranks`) and the
gathered per-rank results (`gather`).  Under torchrun the backend is NCCL on
GPUs; the same calls run on `gloo` for the CPU tests.
"""
from __future__ import annotations

import os
from typing import Sequence


def world() -> tuple[int, int, int]:
    """(world size, rank, local rank) from the torchrun environment."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def shard(items: Sequence, rank: int, world_size: int) -> list:
    """The items of one rank: a round-robin split, so that ranks get systems
    of every size when the items are sorted by size."""
    if world_size < 1 or not 0 <= rank < world_size:
        raise ValueError(f"rank {rank} outside a world of {world_size}")
    return [it for k, it in enumerate(items) if k % world_size == rank]


def shard_by_work(works: Sequence[float], world_size: int) -> list[list[int]]:
    """Indices per rank that balance the summed work (largest first to the
    least-loaded rank); deterministic for equal inputs."""
    load = [0.0] * world_size
    out: list[list[int]] = [[] for _ in range(world_size)]
    for k in sorted(range(len(works)), key=lambda k: (-works[k], k)):
        r = min(range(world_size), key=lambda r: (load[r], r))
        out[r].append(k)
        load[r] += works[k]
    return [sorted(v) for v in out]


def _dist():
    import torch.distributed as dist
    return dist if dist.is_available() and dist.is_initialized() else None


def max_over_ranks(value: float, device=None) -> float:
    """The largest value over all ranks (the job's time is its slowest rank)."""
    dist = _dist()
    if dist is None:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(value: float, device=None) -> float:
    dist = _dist()
    if dist is None:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def gather(obj) -> list:
    """Every rank's object, in rank order, on every rank."""
    dist = _dist()
    if dist is None:
        return [obj]
    out = [None] * dist.get_world_size()
    dist.all_gather_object(out, obj)
    return out


def job_throughput(units_per_rank: Sequence[float], seconds_per_rank: Sequence[float]) -> float:
    """Whole-job rate: all units over the slowest rank's time."""
    return float(sum(units_per_rank)) / max(seconds_per_rank)
