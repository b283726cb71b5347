"""Multi-GPU form of the hot path: replicas.

Samples of one generation are independent, but every generation needs all
updated haplotypes of its chunk, and separate chunks are independent
problems.  So N GPUs run N independent chunks (weak scaling), one process
per GPU, with no collective on the data path: the only collectives are the
barrier around the timed region and the max-over-ranks of the elapsed time.
"""
from __future__ import annotations

import os
from dataclasses import dataclass


@dataclass(frozen=True)
class Replica:
    world: int
    rank: int
    local_rank: int
    data_seed: int      # seed of this rank's synthetic chunk
    rng_seed: int       # key of this rank's counter-based streams


def plan(base_seed: int, rank: int | None = None, world: int | None = None,
         local_rank: int | None = None) -> Replica:
    world = int(os.environ.get("WORLD_SIZE", "1")) if world is None else world
    rank = int(os.environ.get("RANK", "0")) if rank is None else rank
    local_rank = int(os.environ.get("LOCAL_RANK", str(rank))) if local_rank is None \
        else local_rank
    if not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside world of {world}")
    return Replica(world, rank, local_rank, data_seed=base_seed + 1000 * rank,
                   rng_seed=0x9E3779B97F4A7C15 ^ (base_seed + rank))


def max_elapsed(elapsed: float, device=None) -> float:
    """Max of a per-rank elapsed time over all ranks (identity for one)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return elapsed
    t = torch.tensor([elapsed], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
