"""Shot-parallel replicas across processes (one GPU per process).

Shots are independent, so the multi-GPU path has no data exchange: each rank
takes a disjoint subset of the shot list — the reference's round-robin node split
(readmodel.py:121-126, `shotlist[nodei::nnode]`) applied per rank — runs it on
its own GPU and writes its own records.  The only collectives are a barrier and
a max-reduction of the per-rank timings (the job finishes when the slowest rank
does), so weak scaling is the model.
"""
from __future__ import annotations

import os


def env_rank():
    """(world_size, rank, local_rank) from the torchrun environment (1, 0, 0 if unset)."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def shots_for_rank(shots, rank: int, world: int):
    """Round-robin slice of the shot list for one rank, as allocateNode splits nodes."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside world of {world}")
    return list(shots)[rank::world]


def max_over_ranks(value: float, dist=None, device=None) -> float:
    """Maximum of a per-rank scalar (seconds, milliseconds) over all ranks."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(units_per_rank, seconds_per_rank, dist=None, device=None) -> float:
    """Whole-job throughput: all ranks' units over the slowest rank's time."""
    total = float(units_per_rank)
    if dist is not None and dist.is_initialized() and dist.get_world_size() > 1:
        import torch
        t = torch.tensor([total], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.SUM)
        total = float(t.item())
    return total / max_over_ranks(seconds_per_rank, dist, device)
