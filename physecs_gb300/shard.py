"""Scene shards over several GPUs.

The hot path shards at scene granularity: scenes, and serving requests, are
independent, so a workload splits over GPUs with no exchange between them.  One
process drives one GPU; this module decides which scenes or requests each one takes.
"""
from __future__ import annotations

import heapq


def partition(weights, n_parts):
    """Split items (weights = bodies per scene) into n_parts lists of item indices with
    about equal total weight: longest processing time first, each item to the currently
    lightest part (ties: the lower part index; items of equal weight in index order).
    Deterministic, and each part's indices come back sorted."""
    if n_parts < 1:
        raise ValueError("n_parts must be at least 1")
    order = sorted(range(len(weights)), key=lambda i: (-weights[i], i))
    heap = [(0, k) for k in range(n_parts)]
    parts = [[] for _ in range(n_parts)]
    for i in order:
        load, k = heapq.heappop(heap)
        parts[k].append(i)
        heapq.heappush(heap, (load + weights[i], k))
    return [sorted(p) for p in parts]


class Router:
    """Routes a stream of serving requests to per-GPU servers.  Each request goes to the
    shard with the least work routed to it so far (work = bodies x frames; ties: the lower
    shard).  The choice depends only on the requests seen, in order, so every process
    that sees the same stream routes it the same way without talking to the others."""

    def __init__(self, n_shards):
        if n_shards < 1:
            raise ValueError("n_shards must be at least 1")
        self.load = [0] * n_shards

    def route(self, work):
        k = min(range(len(self.load)), key=lambda i: (self.load[i], i))
        self.load[k] += work
        return k
