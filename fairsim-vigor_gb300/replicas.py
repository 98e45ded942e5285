"""Multi-GPU form: independent replicas.

Datasets, channels and live requests are independent units (the reference runs them on
independent threads, org/fairsim/livemode/ReconstructionRunner.java:376-594), so N GPUs run
N replicas with no data-path collective: each rank takes a disjoint share of the units and
the only cross-rank step is timing (max over ranks) for reporting.
"""
from __future__ import annotations


def shard(n_units: int, rank: int, world: int):
    """Unit indices of `rank`: a contiguous, balanced split (sizes differ by at most one)."""
    if world < 1 or not (0 <= rank < world):
        raise ValueError("bad rank/world %d/%d" % (rank, world))
    base, extra = divmod(n_units, world)
    start = rank * base + min(rank, extra)
    return list(range(start, start + base + (1 if rank < extra else 0)))


def max_over_ranks(value: float, device=None) -> float:
    """Max of a per-rank value (elapsed time) over all ranks; identity without a process group."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(value: float, device=None) -> float:
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())
