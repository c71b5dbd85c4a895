"""Sharding batched instances over ranks: the greedy size-balanced partition
(every instance on exactly one rank, loads balanced, the same answer on
every rank) and a world-size-2 gloo run in which each rank simulates its own
shard as one batched network (the oracle stands in for the per-rank engine,
which needs a GPU) and the end-of-run reduction gives the events of the
whole batch, per instance identical to the unsharded run."""
import json
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from neuronbridge_gb300.partition import partition_instances, shard_loads

SMALL = dict(instances=6, lo=40, hi=160)
STEPS = 150


def _port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_partition_covers_every_instance_once():
    from neuronbridge_gb300 import workloads

    sizes, _ = workloads.batched_params(256)
    for world in (1, 2, 3, 4, 8):
        shards = partition_instances(sizes, world)
        assert len(shards) == world
        allk = np.concatenate(shards)
        assert np.array_equal(np.sort(allk), np.arange(256))
        for s in shards:
            assert np.all(np.diff(s) > 0)  # ascending, no repeats
        loads = shard_loads(sizes, shards)
        # greedy longest-first bound: no shard exceeds another by more than one instance
        assert loads.max() - loads.min() <= sizes.max()
        assert loads.sum() == sizes.sum()
        assert partition_instances(sizes, world)[0].tolist() == shards[0].tolist()  # deterministic


def test_partition_small_cases():
    assert [s.tolist() for s in partition_instances([5, 1, 4], 2)] == [[0], [1, 2]]
    assert [s.tolist() for s in partition_instances([3, 3, 3, 3], 2)] == [[0, 2], [1, 3]]
    # fewer instances than ranks: the extra ranks get nothing
    assert [s.tolist() for s in partition_instances([7], 3)] == [[0], [], []]
    assert [s.tolist() for s in partition_instances([], 2)] == [[], []]
    with pytest.raises(ValueError):
        partition_instances([1, 2], 0)
    with pytest.raises(ValueError):
        partition_instances([1, -2], 2)
    with pytest.raises(ValueError):
        partition_instances([1, float("nan")], 2)


def _run_shard(indices):
    """Simulate instances ``indices`` of the small batch as one network in the
    oracle; return (events, {instance: spike raster as lists})."""
    import oracle
    from neuronbridge_gb300 import NetworkDescription, workloads

    if len(indices) == 0:
        return 0, {}
    parts = [workloads.batched_instance(int(k), **SMALL) for k in indices]
    union, first, _ = NetworkDescription.concat(parts)
    o = oracle.OracleNet(union.flat(0.1))
    o.run(STEPS)
    t, i = o.spikes()
    per = {}
    for j, k in enumerate(indices):
        keep = (i >= first[j]) & (i < first[j + 1])
        per[int(k)] = [t[keep].tolist(), (i[keep] - first[j]).tolist()]
    return o.num_events, per


def _rank_main(rank, world, port, out_dir):
    import torch.distributed as dist

    from neuronbridge_gb300 import workloads
    from neuronbridge_gb300.replicas import aggregate

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        sizes, _ = workloads.batched_params(**SMALL)
        mine = partition_instances(sizes, world)[rank]
        events, per = _run_shard(mine)
        times, work = aggregate([1.0 + rank], [events])
        with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as f:
            json.dump({"mine": mine.tolist(), "events": events, "times": times, "work": work, "per": per}, f)
    finally:
        dist.destroy_process_group()


def test_sharded_batch_gloo_world2(tmp_path, oracle_lib):
    from neuronbridge_gb300 import workloads

    world = 2
    mp.spawn(_rank_main, args=(world, _port(), str(tmp_path)), nprocs=world, join=True)
    res = [json.load(open(tmp_path / f"rank{r}.json")) for r in range(world)]
    assert sorted(res[0]["mine"] + res[1]["mine"]) == list(range(SMALL["instances"]))
    assert res[0]["mine"] and res[1]["mine"]
    whole_events, whole = _run_shard(np.arange(SMALL["instances"]))
    for r in res:
        assert r["times"] == [2.0]  # slowest rank's time
        assert r["work"] == [float(whole_events)]  # events of the whole batch
    for r in res:  # each instance's raster does not depend on which shard ran it
        for k, raster in r["per"].items():
            assert raster == whole[int(k)]
    sizes, _ = workloads.batched_params(**SMALL)
    assert sum(len(v[0]) for r in res for v in r["per"].values()) > 0
    assert len(sizes) == SMALL["instances"]
