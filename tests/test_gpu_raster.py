"""Raster ordering on the device: the run call's spike entries, appended by
the update kernel in warp order, come back in (step, id) order through a
per-step spike bitmap.  Checked against the oracle's raster with the default
bitmap budget and with budgets small enough to order a call in chunks of one
and of several steps (NBG_RASTER_BITMAP_WORDS, read at engine creation)."""
import numpy as np
import pytest

import neuronbridge_gb300 as nb
from neuronbridge_gb300 import workloads

pytestmark = pytest.mark.gpu


def _oracle_raster(net, cfg, steps):
    import oracle

    d = net.to_native() if hasattr(net, "to_native") else net
    o = oracle.OracleNet(d.flat(cfg.timestep))
    o.run(steps)
    t, i = o.spikes()
    keep = np.repeat(d.layer_output, d.layer_count)[i]
    t, i = t[keep], i[keep]
    order = np.lexsort((i, t))
    return t[order], i[order]


@pytest.mark.parametrize("budget", [None, 1, 100])
def test_raster_order_matches_oracle(oracle_lib, monkeypatch, budget):
    net, cfg = workloads.plain_lif(n=400, steps=300)
    if budget is not None:
        monkeypatch.setenv("NBG_RASTER_BITMAP_WORDS", str(budget))
    sim = nb.Simulation(net, cfg)
    sim.run(120)
    first = sim.bench_profiling_snapshot()
    sim.run(180)
    snap = sim.bench_profiling_snapshot()
    t, i = sim.spike_raster()
    rt, ri = _oracle_raster(net, cfg, 300)
    assert len(t) > 0
    assert np.array_equal(t, rt) and np.array_equal(i, ri)
    # one chunk of four kernels, or one per chunk of steps (121 updates, then 180)
    wp = ((net.to_native().neuron_count + 31) // 32 + 3) // 4 * 4
    chunk = lambda count: 1 if budget is None else -(-count // max(1, budget // wp))
    assert first["raster_order_launches"] == 4 * chunk(121)
    assert snap["raster_order_launches"] == 4 * chunk(180)
    assert snap["raster_order_ms"] > 0 and snap["raster_download_ms"] >= 0 and snap["raster_append_ms"] >= 0


def test_raster_order_large_batch(oracle_lib):
    """A batch whose raster holds more than 65,536 entries per call equals
    the oracle's raster of the union."""
    singles, union, cfg = workloads.batched_lif(instances=24, lo=500, hi=4000, steps=200)
    sim = nb.Simulation.batch(singles, cfg)
    sim.run(200)
    t, i = sim.spike_raster()
    rt, ri = _oracle_raster(union, cfg, 200)
    assert len(t) > (1 << 16)
    assert np.array_equal(t, rt) and np.array_equal(i, ri)


def test_raster_profile_of_a_silent_call():
    """A run call that records no spike orders nothing and says so."""
    net, cfg = workloads.plain_lif(n=200, steps=50, rate_hz=0.0)
    sim = nb.Simulation(net, cfg)
    sim.run(50)
    snap = sim.bench_profiling_snapshot()
    assert len(sim.spike_raster()[0]) == 0
    assert snap["raster_order_launches"] == 0 and snap["raster_order_ms"] == 0.0


def test_raster_host_fallback_when_device_ordering_fails(oracle_lib, monkeypatch):
    """The step loop has already advanced the engine when the raster is
    ordered, so a failed device ordering (an allocation failure, injected on
    the host with NBG_RASTER_ORDER_FAIL) falls back to ordering the
    downloaded entries on the host: no spike of the call is lost."""
    net, cfg = workloads.plain_lif(n=400, steps=300)
    monkeypatch.setenv("NBG_RASTER_ORDER_FAIL", "1")
    sim = nb.Simulation(net, cfg)
    sim.run(120)
    sim.run(180)
    assert sim.bench_profiling_snapshot()["raster_order_launches"] == -1
    t, i = sim.spike_raster()
    rt, ri = _oracle_raster(net, cfg, 300)
    assert len(t) > 0
    assert np.array_equal(t, rt) and np.array_equal(i, ri)
