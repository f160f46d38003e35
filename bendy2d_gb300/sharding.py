"""World sharding across ranks (one process per GPU).

Worlds share no state, so a multi-GPU run partitions them across ranks and
never exchanges simulation data; only timings (and, optionally, results for
inspection) are gathered.  Assignment balances particle-substeps with the
greedy longest-processing-time rule: heaviest world first, each to the
currently lightest rank.
"""
from __future__ import annotations

import heapq
from typing import Sequence


def shard(costs: Sequence[float], nranks: int) -> list:
    """Return nranks lists of world indices; each world appears exactly once."""
    if nranks < 1:
        raise ValueError("nranks must be >= 1")
    heap = [(0.0, r) for r in range(nranks)]
    out = [[] for _ in range(nranks)]
    for i in sorted(range(len(costs)), key=lambda k: (-costs[k], k)):
        load, r = heapq.heappop(heap)
        out[r].append(i)
        heapq.heappush(heap, (load + float(costs[i]), r))
    for lst in out:
        lst.sort()
    return out


def world_cost(scene) -> float:
    """particle-substeps of one update"""
    return float(scene.n_particles * scene.sub_steps)
