"""Rank-balanced partition of independent Schur updates across GPUs.

The Schur updates of one TLR Cholesky panel are independent: update (i, j)
reads the panel tiles A_i0, A_j0 and its own C_ij and writes only C_ij (the
reference's per-tile call, src/compute/hcore_dgemm.c:703).  Sharding them
across GPUs needs no collective on the data path.  What it needs is balance:
the cost of one update grows with k = a + c (two Householder QRs of M x k,
a Jacobi SVD of order k, two rebuilds), and k runs from 13 to 70 on the
65,536-point panel, so equal update counts leave the rank with the heaviest
share setting the max-over-ranks time.  This module assigns updates by
longest processing time first (each update, heaviest first, to the least
loaded rank) on a per-update FP64 cost model.
"""
from __future__ import annotations

import heapq

# mean Jacobi sweeps per update on the panel workload (the SVD's sweep count
# is data dependent; this only weights the k^3 term of the model)
JACOBI_SWEEPS = 3.7


def update_cost(M: int, a: int, b: int, c: int) -> float:
    """FP64 multiply-adds of one update, as the batched phases execute it:
    the factor products F = AV^T BV and G = BU F^T (2abM), two Householder
    QRs of M x k (M k^2 each), the Jacobi SVD of order k (about 4 k^3 per
    sweep) and two rebuilds (2 M k r each, with the new rank r, unknown
    before the update runs, taken as k / 2)."""
    k = a + c
    return 2.0 * a * b * M + 2.0 * M * k * k + JACOBI_SWEEPS * 4.0 * k ** 3 + 2.0 * M * k * k


def lpt_partition(costs, world: int) -> list:
    """Longest-processing-time-first assignment of items with the given
    costs to `world` ranks.  Returns, per rank, the list of item indices in
    increasing order.  Deterministic (ties by item index, then rank)."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(costs)), key=lambda u: (-float(costs[u]), u))
    heap = [(0.0, r) for r in range(world)]
    parts = [[] for _ in range(world)]
    for u in order:
        load, r = heapq.heappop(heap)
        parts[r].append(u)
        heapq.heappush(heap, (load + float(costs[u]), r))
    return [sorted(p) for p in parts]


def imbalance(costs, parts) -> float:
    """Heaviest rank's load over the mean load, minus one (0 = perfect)."""
    loads = [sum(float(costs[u]) for u in p) for p in parts]
    mean = sum(loads) / len(loads)
    return max(loads) / mean - 1.0 if mean > 0 else 0.0


def tiles_read(updates) -> set:
    """Tiles that a list of panel-0 updates (i, j) reads: A_i0, A_j0, C_ij."""
    need = set()
    for i, j in updates:
        need.update(((i, 0), (j, 0), (i, j)))
    return need
