"""Timing aggregation for a run on several GPUs.

The simulation step does not shard: every rank simulates an independent
replica of the network and nothing crosses between ranks on the data path.
A multi-GPU run is therefore N replicas; its time is the slowest rank's and
its work (synaptic events) is the sum over ranks.  The only collective is
this end-of-run reduction of a few scalars.
"""
from __future__ import annotations


def aggregate(times, work, device=None):
    """Return (max over ranks of each entry of ``times``, sum over ranks of
    each entry of ``work``).  Without an initialised process group, or with
    one rank, the inputs come back unchanged."""
    import torch
    import torch.distributed as dist

    times, work = [float(x) for x in times], [float(x) for x in work]
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return times, work
    t = torch.tensor(times, dtype=torch.float64, device=device)
    w = torch.tensor(work, dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(w, op=dist.ReduceOp.SUM)
    return t.tolist(), w.tolist()
