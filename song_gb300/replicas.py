"""Host logic of the multi-GPU run: one replica of the index per GPU.

Queries are independent (one warp per query, warp_astar_accelerator.h:48,386),
so N GPUs run N replicas with no data-path collective: every rank searches its
own copy of the query set on its own copy of the index.  The only exchange is
the timing: the job's time is the slowest rank's, and the job's rate counts
the queries of all ranks."""
from __future__ import annotations


def max_over_ranks(x: float, dist=None, device: str = "cpu") -> float:
    """The largest x over all ranks of the default process group (x itself
    without one).  device: where the reduction tensor lives (cuda for NCCL,
    cpu for gloo)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank: int, steps: int, world: int, slowest_seconds: float) -> float:
    """Units per second of the whole job: all ranks' units over the slowest
    rank's time."""
    return world * units_per_rank * steps / slowest_seconds
