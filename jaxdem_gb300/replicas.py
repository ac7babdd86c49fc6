"""Replica bookkeeping for multi-GPU runs.

The step shards only as replicas: independent systems (or independent copies
of one workload) per rank, with no exchange step and no collective on the data
path.  The only collective is the timing reduction of a benchmark, the
maximum over ranks of each rank's elapsed time, so the aggregate throughput is
the work of all ranks over the slowest rank's time.
"""

from __future__ import annotations

from typing import Optional, Sequence


def max_over_ranks(dist, value: float, device: Optional[str] = None) -> float:
    """Maximum of `value` over the ranks of the default process group (any backend;
    `device` is where the reduction tensor lives, e.g. "cuda:0" for NCCL, None for gloo)."""
    if dist is None:
        return float(value)
    import torch

    t = torch.tensor([float(value)], dtype=torch.float64, device=device or "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def shard(n_items: int, rank: int, world: int) -> range:
    """Contiguous block of the items owned by `rank` (sizes differ by at most one)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank must lie in [0, world)")
    base, extra = divmod(int(n_items), int(world))
    start = rank * base + min(rank, extra)
    return range(start, start + base + (1 if rank < extra else 0))


def aggregate_throughput(units_per_rank: Sequence[int], max_seconds: float) -> float:
    """Whole-job throughput: the units every rank processed over the slowest rank's time."""
    return float(sum(units_per_rank)) / float(max_seconds)
