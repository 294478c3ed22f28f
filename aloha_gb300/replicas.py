"""Multi-GPU form: replicas only.

Views are independent, so N processes (one per GPU) each hold the whole
volume and render views r, r+N, r+2N, ... with no exchange on the data path;
only the timing and the sample totals are reduced (max of the elapsed times,
sum of the samples).  The reference's image exchange (IceT over MPI) has no
counterpart because all virtual ranks of a frame share one GPU's memory.
"""
from __future__ import annotations


def shard_views(n_views: int, rank: int, world: int) -> list[int]:
    """The views process `rank` of `world` renders (round robin)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("need 0 <= rank < world")
    return list(range(rank, n_views, world))


def _reduce(value: float, op: str, device=None) -> float:
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX if op == "max" else dist.ReduceOp.SUM)
    return float(t.item())


def max_over_ranks(value: float, device=None) -> float:
    """Slowest rank's value (the whole job ends when the last replica does)."""
    return _reduce(value, "max", device)


def sum_over_ranks(value: float, device=None) -> float:
    return _reduce(value, "sum", device)
