"""Edge cases of the step engine, bit-exact against the oracle: no synapses,
in-degree above the fast path's 1,024 (the general drain), more than 32
inline generator inputs, a one-step minimum delay (one step per launch),
very long delays, and the raster capacity error."""
import numpy as np
import pytest

import neuronbridge_gb300 as nb
from neuronbridge_gb300 import Connection, Network, NeuronLayer, SimulationConfig, float32
from neuronbridge_gb300.workloads import LIF_PARAMS

pytestmark = pytest.mark.gpu


def _lif(n, **kw):
    return NeuronLayer("TimeDrivenLIF_Voltage_jump", n, parameters=dict(LIF_PARAMS, **kw.pop("params", {})), **kw)


def _check(net, cfg, steps, **sim_kw):
    import oracle

    sim = nb.Simulation(net, cfg, **sim_kw)
    sim.run(steps)
    o = oracle.OracleNet(net.to_native().flat(cfg.timestep))
    o.run(steps)
    d = net.to_native()
    keep = np.repeat(d.layer_output, d.layer_count)
    t, i = o.spikes()
    t, i = t[keep[i]], i[keep[i]]
    order = np.lexsort((i, t))
    st, si = sim.spike_raster()
    assert np.array_equal(st, t[order]) and np.array_equal(si, i[order])
    assert np.array_equal(sim.state_field(0), o.state(0).astype(np.float32))
    assert sim.num_events == o.num_events
    return sim


def test_no_synapses_constant_current(oracle_lib):
    net = Network().add_layer(_lif(64, output=True, params={"I_ext": float32(20.0)}))
    sim = _check(net, SimulationConfig(steps=3000, timestep=0.1), 3000)
    assert len(sim.spike_raster()[0]) > 0 and sim.num_events == 0


def test_in_degree_above_fast_path(oracle_lib):
    """Targets with 1,500 in-synapses (47 mask words) drain through the
    general path; sources are LIF neurons driven by Poisson generators."""
    rng = np.random.default_rng(4)
    net = Network()
    net.add_layer(_lif(2000))
    net.add_layer(_lif(20, output=True))
    net.add_layer(NeuronLayer.poisson_rate(2000, rate_bias_hz=6000.0, rate_gain_hz_per_current=0.0))
    ids = np.arange(2000, dtype=np.int32)
    net.connect(Connection(ids + 2020, ids, weight=0.6, delay=1))
    src = np.concatenate([rng.choice(2000, 1500, replace=False) for _ in range(20)]).astype(np.int32)
    tgt = np.repeat(np.arange(2000, 2020), 1500).astype(np.int32)
    typ = (rng.random(len(src)) < 0.2).astype(np.int32)
    net.connect(Connection(src, tgt, synapse_type=typ, weight=0.05, delay=rng.integers(2, 9, len(src)).astype(np.int32)))
    sim = _check(net, SimulationConfig(steps=1500, timestep=0.1), 1500)
    assert np.any(sim.spike_raster()[1] >= 2000)


def test_many_generator_inputs(oracle_lib):
    """40 inline Poisson generator inputs per target (> 32: general path)."""
    net = Network()
    net.add_layer(_lif(50, output=True))
    net.add_layer(NeuronLayer.poisson_rate(400, rate_bias_hz=900.0, rate_gain_hz_per_current=0.0))
    rng = np.random.default_rng(5)
    src = (50 + np.concatenate([rng.choice(400, 40, replace=False) for _ in range(50)])).astype(np.int32)
    tgt = np.repeat(np.arange(50), 40).astype(np.int32)
    net.connect(Connection(src, tgt, weight=1.2, delay=rng.integers(1, 4, len(src)).astype(np.int32)))
    sim = _check(net, SimulationConfig(steps=2000, timestep=0.1), 2000)
    assert len(sim.spike_raster()[0]) > 0


def test_one_step_delay_and_long_delays(oracle_lib):
    """Recurrent delay 1 (B = 1: one step per launch) next to 3,000-step
    delays (a 3,001-slot ring)."""
    rng = np.random.default_rng(6)
    net = Network()
    net.add_layer(_lif(300, output=True))
    net.add_layer(NeuronLayer.poisson_rate(300, rate_bias_hz=7000.0, rate_gain_hz_per_current=0.0))
    ids = np.arange(300, dtype=np.int32)
    net.connect(Connection(ids + 300, ids, weight=0.5, delay=1))
    s, t = rng.integers(0, 300, 3000).astype(np.int32), rng.integers(0, 300, 3000).astype(np.int32)
    net.connect(Connection(s, t, weight=0.4, delay=np.where(rng.random(3000) < 0.5, 1, 3000).astype(np.int32)))
    sim = _check(net, SimulationConfig(steps=7000, timestep=0.1), 7000)
    assert sim.block_steps == 1


def test_raster_capacity_overflow_is_an_error():
    net = Network().add_layer(_lif(64, output=True, params={"I_ext": float32(20.0)}))
    sim = nb.Simulation(net, SimulationConfig(steps=3000, timestep=0.1), spike_capacity=10)
    with pytest.raises(nb.NbgError, match="capacity"):
        sim.run(3000)
