"""Batches of independent structures (MD snapshots or configurations).

Structures are independent, so a multi-GPU job shards them across ranks with
no data-path collective; only the bookkeeping (totals, timings) is reduced.
The three-center work of a structure grows with its atom count times the
square of its density (common-neighbor triplets per atom scale with the
number of neighbors squared), so structures of 32 to 512 atoms differ in
cost by far more than their atom counts.  With weights, `shard` balances the
ranks by the greedy longest-first rule: items in decreasing weight, each to
the rank with the least load so far, which keeps the largest load within
4/3 of the best possible split.
"""
from __future__ import annotations

import numpy as np


def work_estimate(ratom, lattice):
    """Relative three-center work of a periodic structure: N * (N / V)^2."""
    n = len(ratom)
    vol = abs(float(np.linalg.det(np.asarray(lattice, np.float64))))
    dens = n / vol if vol > 0 else 1.0
    return n * dens * dens


def shard(n_items, rank, world, weights=None):
    """Indices (ascending) of the items rank `rank` of `world` assembles.
    Without weights: every world-th item.  With weights (one per item):
    longest-first greedy assignment to the least-loaded rank (ties go to
    the lower rank, then the lower item index), so every rank computes the
    same partition."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank/world %d/%d" % (rank, world))
    if weights is None:
        return list(range(rank, n_items, world))
    w = np.asarray(weights, np.float64)
    if len(w) != n_items or (w < 0).any():
        raise ValueError("need one non-negative weight per item")
    order = sorted(range(n_items), key=lambda i: (-w[i], i))
    load = np.zeros(world)
    mine = []
    for i in order:
        r = int(np.argmin(load))
        load[r] += w[i]
        if r == rank:
            mine.append(i)
    return sorted(mine)
