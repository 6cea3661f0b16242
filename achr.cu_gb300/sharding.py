"""Chains over ranks: one process per GPU, each sampling its own block of chain ids.

Chains are independent and every random draw is keyed by (seed, chain id, step,
attempt), so a rank that samples chain ids [offset, offset + count) produces
exactly the columns a single process would produce for those ids.  The data
path therefore has no collective; the only collectives are the barrier around
the timed region and the maximum of the per-rank times (the job is as slow as
its slowest rank).  The reference runs one process on one GPU (its chains are
ACHRcu/ACHRCuda.cu:741's grid over nPoints); this is the weak-scaling split of
the same chain ids.
"""
from __future__ import annotations


def chain_block(rank: int, world: int, chains_per_rank: int) -> tuple[int, int]:
    """(first chain id, chain count) of `rank` when every rank runs chains_per_rank chains."""
    if not 0 <= rank < world or chains_per_rank < 0:
        raise ValueError("bad rank, world size or chain count")
    return rank * chains_per_rank, chains_per_rank


def split_chains(rank: int, world: int, total: int) -> tuple[int, int]:
    """(first chain id, chain count) of `rank` when `total` chains are split as evenly as possible."""
    if not 0 <= rank < world or total < 0:
        raise ValueError("bad rank, world size or chain count")
    base, extra = divmod(total, world)
    count = base + (1 if rank < extra else 0)
    offset = rank * base + min(rank, extra)
    return offset, count


def max_over_ranks(value: float, device=None) -> float:
    """Maximum of a per-rank scalar (a timed region) over the process group."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
