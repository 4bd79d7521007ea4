"""Replica sharding of independent induced-dipole solves over ranks.

Snapshots (and their right-hand sides) are independent linear systems, so a
batched workload shards by snapshot with no collective on the data path: rank
r of W solves snapshots r, r + W, r + 2W, ... on its own GPU, and the results
are gathered once at the end.  A single system is never split across ranks
(one GPU holds the largest system many times over), so there is no halo or
multipole exchange.  Works with any torch.distributed backend (gloo on CPU,
nccl on GPUs); without an initialised process group it runs everything
locally.
"""
from __future__ import annotations

from typing import Callable, Dict, List, Sequence


def shard(n_items: int, rank: int, world: int) -> List[int]:
    """Items owned by `rank`: round-robin, so uneven snapshot sizes spread out."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"invalid rank {rank} of world {world}")
    return list(range(rank, n_items, world))


def _dist():
    try:
        import torch.distributed as dist
    except ImportError:  # pragma: no cover - torch is a dependency
        return None
    return dist if dist.is_available() and dist.is_initialized() else None


def solve_sharded(items: Sequence, solve_one: Callable, gather: bool = True) -> Dict[int, object]:
    """Solves `solve_one(item)` for this rank's share of `items`.

    Returns {index: result} for this rank's items, or for all items when
    `gather` is set (one all_gather of the results after every solve is done).
    """
    dist = _dist()
    rank, world = (dist.get_rank(), dist.get_world_size()) if dist else (0, 1)
    local = {i: solve_one(items[i]) for i in shard(len(items), rank, world)}
    if not gather or dist is None:
        return local
    parts: List[Dict[int, object]] = [None] * world  # type: ignore[list-item]
    dist.all_gather_object(parts, local)
    out: Dict[int, object] = {}
    for p in parts:
        overlap = out.keys() & p.keys()
        if overlap:
            raise RuntimeError(f"items solved twice: {sorted(overlap)}")
        out.update(p)
    if len(out) != len(items):
        raise RuntimeError(f"gathered {len(out)} results for {len(items)} items")
    return out
