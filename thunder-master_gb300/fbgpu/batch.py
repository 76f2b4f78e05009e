"""Batches of independent structures (MD snapshots or configurations).

Structures are independent, so a multi-GPU job shards them across ranks with
no data-path collective: rank r takes every world-th structure, in order.
Only the bookkeeping (totals, timings) is reduced.
"""
from __future__ import annotations


def shard(n_items, rank, world):
    """Indices of the items rank `rank` of `world` assembles."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank/world %d/%d" % (rank, world))
    return list(range(rank, n_items, world))
