"""Sharding independent scenes across GPUs (one process per GPU).

Scenes of a sweep are independent, so the multi-GPU form needs no exchange in
the data path: each rank advances its own share of the scenes as one batch,
and only the timing (max over ranks) and the final metrics are gathered on
the host.  The share is a particle-count-balanced partition: longest
processing time first (Graham 1969, "Bounds on multiprocessing timing
anomalies") - scenes in decreasing particle count, each to the currently
lightest rank - whose heaviest rank is within one scene of the mean load
(max load <= mean + max scene).
"""
from __future__ import annotations

import heapq


def balanced_partition(weights, n_parts: int) -> list[list[int]]:
    """Indices of `weights` split into n_parts lists (each sorted), balanced
    by total weight; ties go to the lower part index, so every rank computes
    the same partition."""
    if n_parts < 1:
        raise ValueError("n_parts must be >= 1")
    heap = [(0, r) for r in range(n_parts)]
    parts: list[list[int]] = [[] for _ in range(n_parts)]
    order = sorted(range(len(weights)), key=lambda i: (-weights[i], i))
    for i in order:
        load, r = heapq.heappop(heap)
        parts[r].append(i)
        heapq.heappush(heap, (load + weights[i], r))
    return [sorted(p) for p in parts]


def loads(weights, parts) -> list[int]:
    return [sum(weights[i] for i in p) for p in parts]
