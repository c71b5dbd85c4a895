"""Sharding independent network instances over ranks.

Instances of a batch (networks with no connection between them) are the
unit that shards: each rank builds one batched engine over its own share
and nothing crosses between ranks on the data path.  The share is chosen by
greedy size-balanced bin packing (longest processing time first): instances
in decreasing order of work, each given to the rank with the least work so
far.  The work of an instance is its synapse count when known, else its
neuron count (the delivery pass dominates the step and the batched
workloads have a fixed in-degree).  Ties go to the lower instance index and
the lower rank, so every rank computes the same partition on its own.

Results per instance do not depend on the partition: an instance's
connectivity and its PoissonRate hash stream are keyed by its own local ids,
so instance k run in any shard equals instance k run in the whole batch.
"""
from __future__ import annotations

import numpy as np


def partition_instances(work, world: int) -> list[np.ndarray]:
    """Split instances 0..len(work)-1 over ``world`` ranks.  Returns one
    ascending int64 index array per rank (possibly empty when there are
    fewer instances than ranks); together they cover every instance once."""
    w = np.asarray(work, dtype=np.float64).reshape(-1)
    if world < 1:
        raise ValueError("world size must be >= 1")
    if np.any(~np.isfinite(w)) or np.any(w < 0):
        raise ValueError("instance work must be finite and non-negative")
    order = np.lexsort((np.arange(len(w)), -w))  # work descending, index ascending
    load = np.zeros(world, dtype=np.float64)
    owner = np.empty(len(w), dtype=np.int64)
    for k in order:
        r = int(np.argmin(load))  # first rank among the least loaded
        owner[k] = r
        load[r] += w[k]
    return [np.nonzero(owner == r)[0].astype(np.int64) for r in range(world)]


def shard_loads(work, shards) -> np.ndarray:
    """Total work of each shard."""
    w = np.asarray(work, dtype=np.float64).reshape(-1)
    return np.array([w[s].sum() for s in shards], dtype=np.float64)
