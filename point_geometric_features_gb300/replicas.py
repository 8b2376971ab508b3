"""Host-side logic for running the path on several GPUs, one process each.

The neighbour search and the feature passes have no cross-point exchange:
every query row depends only on the (replicated) cloud and its own index, so
N GPUs either serve N independent workloads (weak scaling: independent
clouds or request streams per rank) or split one cloud's query rows into N
contiguous ranges over a replicated grid and concatenate the row blocks on
the host. No collective is on the data path; the only collective is the
max-over-ranks reduction of the timed region.
"""

from __future__ import annotations

import os

__all__ = ["dist_env", "query_range", "partition_clouds", "max_over_ranks"]


def dist_env() -> tuple[int, int, int]:
    """(rank, world_size, local_rank) from the torchrun environment (1 process: 0, 1, 0)."""
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world < 1 or not (0 <= rank < world) or local < 0:
        raise ValueError(f"inconsistent torchrun environment: rank={rank} world={world} local={local}")
    return rank, world, local


def query_range(m: int, rank: int, world: int) -> tuple[int, int]:
    """Contiguous row range [lo, hi) of `m` query rows owned by `rank`.

    Ranges are disjoint, cover [0, m) in rank order and differ in size by at
    most one row, so concatenating the ranks' row blocks in rank order gives
    the one-GPU result row for row."""
    if world < 1 or not (0 <= rank < world) or m < 0:
        raise ValueError(f"bad shard request: m={m} rank={rank} world={world}")
    base, extra = divmod(m, world)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def partition_clouds(sizes, world: int) -> list[list[int]]:
    """Split independent clouds (by point count) over `world` ranks.

    Longest-processing-time greedy: clouds in decreasing size go to the rank
    with the fewest points so far (ties to the lower rank); each rank's list
    keeps the clouds' original order. Deterministic for a given input."""
    if world < 1:
        raise ValueError("world must be >= 1")
    sizes = [int(s) for s in sizes]
    if any(s < 0 for s in sizes):
        raise ValueError("cloud sizes must be >= 0")
    load = [0] * world
    owner = [0] * len(sizes)
    for i in sorted(range(len(sizes)), key=lambda j: (-sizes[j], j)):
        r = min(range(world), key=lambda q: (load[q], q))
        owner[i] = r
        load[r] += sizes[i]
    return [[i for i in range(len(sizes)) if owner[i] == r] for r in range(world)]


def max_over_ranks(value: float, device=None) -> float:
    """Max of a per-rank float over the default process group (the timed
    region's duration); the value itself when no group is initialised."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
