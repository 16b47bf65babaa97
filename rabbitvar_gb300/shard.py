"""Region sharding across GPUs (one process per GPU).

Regions are independent in the reference (one region per OpenMP task,
src/modes/simpleMode.cpp:320-347), so the multi-GPU form partitions them with
no data-path collective: each rank calls its share and the host concatenates
the record text.  Tumor and normal of one region stay on the same rank.
"""
from __future__ import annotations

import heapq

import numpy as np


def estimate_reads(pos: np.ndarray, regions: list[tuple[int, int]], max_span: int = 1000) -> list[int]:
    """Reads whose start lies in [start - max_span, end] for each region
    (coordinate-sorted 0-based positions); a cheap load estimate."""
    out = []
    for a, b in regions:
        lo = np.searchsorted(pos, a - 1 - max_span, side="left")
        hi = np.searchsorted(pos, b, side="left")
        out.append(int(hi - lo))
    return out


def partition(weights: list[int], n: int) -> list[list[int]]:
    """Longest-processing-time greedy assignment of region indexes to n
    shards; deterministic (ties by index), every region in exactly one shard,
    each shard's list in ascending region order."""
    if n <= 0:
        raise ValueError("n must be positive")
    order = sorted(range(len(weights)), key=lambda i: (-weights[i], i))
    heap = [(0, k) for k in range(n)]
    shards: list[list[int]] = [[] for _ in range(n)]
    for i in order:
        load, k = heapq.heappop(heap)
        shards[k].append(i)
        heapq.heappush(heap, (load + max(weights[i], 1), k))
    return [sorted(s) for s in shards]


def shard_regions(regions, weights, rank: int, world: int):
    idx = partition(weights, world)[rank]
    return [regions[i] for i in idx], idx
