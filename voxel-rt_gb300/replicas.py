"""Multi-GPU as replicas: every rank holds its own copy of the world and renders its
own frames or its share of a camera list; nothing on the data path is exchanged.
The only cross-rank traffic is the timing reduction (max over ranks) used to report
whole-job throughput."""
from __future__ import annotations


def share(n_items: int, rank: int, world_size: int) -> list[int]:
    """Round-robin share of n_items (cameras, requests) for one rank."""
    return list(range(rank, n_items, world_size))


def max_over_ranks(value: float, dist=None, device=None) -> float:
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank: list[int] | int, max_seconds: float, world_size: int = 1) -> float:
    """Units per second of the whole job: all ranks' units over the slowest rank's time."""
    total = sum(units_per_rank) if isinstance(units_per_rank, list) else units_per_rank * world_size
    return total / max_seconds
