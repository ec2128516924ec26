"""Sharding of independent instances across GPUs (one process per GPU).

Instances of a batch share nothing, so N GPUs split them with no data-path
collective: every rank computes the same greedy longest-processing-time
assignment from the instance weights (nonzeros plus variables, a proxy for
the work per iteration) and solves its own share in one persistent launch;
only the timings are combined (max over ranks)."""
from __future__ import annotations

import heapq

import numpy as np


def lpt_partition(weights, parts: int) -> list[list[int]]:
    """Greedy LPT: instances in decreasing weight go to the least loaded part.
    Deterministic (ties broken by part index), so every rank computes the same
    assignment without communicating."""
    if parts < 1:
        raise ValueError("parts must be >= 1")
    w = np.asarray(weights, dtype=np.float64)
    order = sorted(range(len(w)), key=lambda i: (-w[i], i))
    heap = [(0.0, p) for p in range(parts)]
    out: list[list[int]] = [[] for _ in range(parts)]
    for i in order:
        load, p = heapq.heappop(heap)
        out[p].append(i)
        heapq.heappush(heap, (load + w[i], p))
    for p in out:
        p.sort()
    return out


def assemble(parts: list[list[int]], shard_results: list[list]) -> list:
    """Per-rank results (rank r's list in the order of parts[r]) back in the
    batch's instance order."""
    n = sum(len(p) for p in parts)
    out: list = [None] * n
    for idx, res in zip(parts, shard_results):
        if len(idx) != len(res):
            raise ValueError("a rank returned a different number of results than it was assigned")
        for i, r in zip(idx, res):
            out[i] = r
    return out


def instance_weight(d) -> float:
    rp, ci, v, (m, n) = d.csr()
    return float(ci.shape[0] + n)
