"""Partition a batch of chains over data-parallel ranks.

Chains are independent in both layers (no exchange in the forward or backward),
so multi-GPU work is pure batch sharding.  The cost of a chain is linear in its
length, so chains are assigned longest-first to the currently lightest rank
(LPT greedy), which keeps the per-rank residue counts within one chain of each
other.
"""
from __future__ import annotations

import heapq
from typing import Sequence


def partition_chains(lengths: Sequence[int], world_size: int) -> list[list[int]]:
    """Chain indices for each rank, each list sorted ascending."""
    if world_size < 1:
        raise ValueError("world_size must be >= 1")
    heap = [(0, r) for r in range(world_size)]
    parts: list[list[int]] = [[] for _ in range(world_size)]
    order = sorted(range(len(lengths)), key=lambda i: (-int(lengths[i]), i))
    for i in order:
        load, r = heapq.heappop(heap)
        parts[r].append(i)
        heapq.heappush(heap, (load + int(lengths[i]), r))
    return [sorted(p) for p in parts]


def shard_for_rank(lengths: Sequence[int], rank: int, world_size: int) -> list[int]:
    return partition_chains(lengths, world_size)[rank]
