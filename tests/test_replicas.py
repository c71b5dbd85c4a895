"""Multi-GPU runs are independent replicas (the step has no exchange between
ranks).  World-size-2 gloo runs on the CPU check the end-of-run reduction
that bench.py uses: job time = max over ranks, events = sum over ranks, and
that two replicas of the same seeded network do the same work (here with
the oracle standing in for the per-rank engine, which needs a GPU)."""
import json
import os
import socket

import numpy as np
import torch.multiprocessing as mp


def _port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    import torch.distributed as dist

    import oracle
    from neuronbridge_gb300 import workloads
    from neuronbridge_gb300.replicas import aggregate

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        net, cfg = workloads.plain_lif(n=300, steps=200)
        o = oracle.OracleNet(net.to_native().flat(cfg.timestep))
        o.run(200)
        events = float(o.num_events)
        times, work = aggregate([1.0 + rank, 10.0 * (rank + 1)], [events, rank + 1.0])
        with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as f:
            json.dump({"times": times, "work": work, "local_events": events}, f)
    finally:
        dist.destroy_process_group()


def test_replica_aggregation_gloo_world2(tmp_path, oracle_lib):
    world = 2
    mp.spawn(_rank_main, args=(world, _port(), str(tmp_path)), nprocs=world, join=True)
    res = [json.load(open(tmp_path / f"rank{r}.json")) for r in range(world)]
    assert res[0]["local_events"] == res[1]["local_events"] > 0  # same seeded replica
    for r in res:  # every rank sees the same reduced values
        assert r["times"] == [2.0, 20.0]
        assert r["work"] == [2 * res[0]["local_events"], 3.0]


def test_single_process_is_identity():
    from neuronbridge_gb300.replicas import aggregate

    assert aggregate([1.5, 2.5], [7]) == ([1.5, 2.5], [7.0])
    assert np.isfinite(aggregate([0.0], [0.0])[0][0])
