"""Distribution of independent basins over ranks (one GPU per rank).

Basins of an ensemble share nothing during a step, so a multi-GPU run gives
every rank a subset of the basins and needs no exchange in the data path:
each rank advances its own basins; the only collectives are the barriers
and the max-over-ranks of the timed region around a benchmark, and an
optional gather of results for checking.  A single basin split over
ranks, with the reference's halo exchange (mod_xc_mp.h), is the other
multi-rank path: hycadv.decomp.
"""
from __future__ import annotations


def shard(work, world_size: int):
    """Longest-processing-time assignment of items with the given work
    (e.g. cells*layers*tracers) to world_size ranks: items in decreasing
    work, each to the least loaded rank (ties: lowest rank).  Returns one
    list of item indices per rank, each in increasing order."""
    if world_size < 1:
        raise ValueError("world_size must be >= 1")
    load = [0.0] * world_size
    out = [[] for _ in range(world_size)]
    order = sorted(range(len(work)), key=lambda i: (-float(work[i]), i))
    for i in order:
        r = min(range(world_size), key=lambda q: (load[q], q))
        out[r].append(i)
        load[r] += float(work[i])
    return [sorted(x) for x in out]


def imbalance(work, parts) -> float:
    """max rank load / mean rank load (1.0 = perfect balance)."""
    loads = [sum(float(work[i]) for i in p) for p in parts]
    mean = sum(loads) / max(len(loads), 1)
    return max(loads) / mean if mean > 0 else 1.0
