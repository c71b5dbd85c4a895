"""External inputs fused into the device step loop, bit-exact against the
oracle: spikes of input-spike neurons (Simulation.add_external_spikes) and
currents of input-current neurons over current synapses
(Simulation.add_external_currents), in the reference's semantics
(ArrayInputSpikeDriver.cpp, InputSpike.cpp, ArrayInputCurrentDriver.cpp,
InputCurrent.cpp, PropogatedCurrent.cpp, CurrentSynapse totals)."""
import numpy as np
import pytest

import neuronbridge_gb300 as nb
from neuronbridge_gb300 import Connection, LearningRule, Network, NeuronLayer, SimulationConfig, float32
from neuronbridge_gb300.workloads import LIF_PARAMS

pytestmark = pytest.mark.gpu

N_IN, N_CUR, N_LIF = 64, 8, 600


def _network(seed=0, currents=True):
    """input spikes -> LIF (plastic, delays 3..8), LIF -> LIF (delays 3..12),
    input currents -> LIF over current synapses (some targets get two)."""
    rng = np.random.default_rng(seed)
    net = Network()
    net.add_layer(NeuronLayer.input_spike(N_IN, output=True))
    net.add_layer(NeuronLayer.input_current(N_CUR))
    lif0 = N_IN + N_CUR
    params = dict(LIF_PARAMS, t_ref=nb.int32(5))
    net.add_layer(NeuronLayer("TimeDrivenLIF_Voltage_jump", N_LIF, output=True, parameters=params))
    net.add_learning_rule(LearningRule("STDP", {"Max_LTP": float32(0.05), "LTP_tau": float32(16.8),
                                                "Max_LTD": float32(0.06), "LTD_tau": float32(33.1)}))
    src = np.repeat(np.arange(N_IN), 40)
    tgt = lif0 + rng.integers(0, N_LIF, size=len(src))
    net.connect(Connection(src.astype(np.int32), tgt.astype(np.int32), synapse_type=0, weight=4.0,
                           max_weight=8.0, delay=rng.integers(3, 9, size=len(src)).astype(np.int32),
                           synapse_rule=0))
    m = rng.random((N_LIF, N_LIF)) < 0.05
    np.fill_diagonal(m, False)
    s, t = np.nonzero(m)
    inh = s >= int(0.8 * N_LIF)
    net.connect(Connection((lif0 + s).astype(np.int32), (lif0 + t).astype(np.int32),
                           synapse_type=inh.astype(np.int32), weight=np.where(inh, 2.0, 1.5).astype(np.float32),
                           delay=rng.integers(3, 13, size=len(s)).astype(np.int32)))
    if currents:
        cs = np.repeat(np.arange(N_CUR), 60)
        ct = lif0 + rng.integers(0, N_LIF, size=len(cs))
        net.connect(Connection((N_IN + cs).astype(np.int32), ct.astype(np.int32), synapse_type=3, weight=1.0,
                               delay=rng.integers(1, 4, size=len(cs)).astype(np.int32)))
    return net, SimulationConfig(steps=400, timestep=0.1)


def _events(seed=1, t_lo=0, t_hi=400, n=300):
    rng = np.random.default_rng(seed)
    pairs = {(int(t), int(i)) for t, i in zip(rng.integers(t_lo, t_hi, n), rng.integers(0, N_IN, n))}
    t, i = np.array(sorted(pairs)).T
    perm = rng.permutation(len(t))  # unsorted input order
    return t[perm], i[perm]


def _currents(seed=2, t_lo=0, t_hi=400, n=40):
    rng = np.random.default_rng(seed)
    return (rng.integers(t_lo, t_hi, n), N_IN + rng.integers(0, N_CUR, n),
            rng.uniform(5.0, 40.0, n).astype(np.float32))


def _oracle(net, cfg):
    import oracle

    return oracle.OracleNet(net.to_native().flat(cfg.timestep))


def _raster_of(o, net):
    d = net.to_native()
    keep = np.repeat(d.layer_output, d.layer_count)
    t, i = o.spikes()
    t, i = t[keep[i]], i[keep[i]]
    order = np.lexsort((i, t))
    return t[order], i[order]


def _same(sim, o, net):
    (ta, ia), (tb, ib) = sim.spike_raster(), _raster_of(o, net)
    assert len(ta) == len(tb) and np.array_equal(ta, tb) and np.array_equal(ia, ib)
    assert np.array_equal(sim.state_field(0), o.state(0).astype(np.float32))
    assert np.array_equal(sim.state_field(4), o.state(4).astype(np.float32))
    assert np.array_equal(sim.weights()["weight"], o.weights()[0].astype(np.float32))
    assert sim.num_events == o.num_events


@pytest.mark.parametrize("use_graph", [True, False])
def test_external_spikes_bit_exact(oracle_lib, use_graph):
    net, cfg = _network(currents=False)
    sim = nb.Simulation(net, cfg, use_graph=use_graph)
    o = _oracle(net, cfg)
    t, i = _events()
    sim.add_external_spikes(t, i)
    o.add_external_spikes(t, i)
    sim.run(150)  # events after this call stay pending
    o.run(150)
    _same(sim, o, net)
    t2, i2 = _events(seed=5, t_lo=160, t_hi=600)  # added between calls
    sim.add_external_spikes(t2, i2)
    o.add_external_spikes(t2, i2)
    sim.run(250)
    sim.run(200)
    o.run(250)
    o.run(200)
    _same(sim, o, net)
    st, si = sim.spike_raster()
    inputs = si < N_IN
    assert inputs.sum() == len(t) + len(t2)  # every external spike is in the raster (output layer)
    assert (~inputs).sum() > 0
    assert not np.array_equal(sim.weights()["weight"], net.to_native().weight)  # pre STDP ran


def test_external_currents_and_spikes_bit_exact(oracle_lib):
    net, cfg = _network()
    sim = nb.Simulation(net, cfg)
    o = _oracle(net, cfg)
    t, i = _events()
    ct, ci, cv = _currents()
    # one source sends twice at the same step: the later value wins
    ct = np.concatenate([ct, [50, 50]])
    ci = np.concatenate([ci, [N_IN + 1, N_IN + 1]])
    cv = np.concatenate([cv, [30.0, -20.0]]).astype(np.float32)
    for s in (sim, o):
        s.add_external_spikes(t, i)
        s.add_external_currents(ct, ci, cv)
    sim.run(400)
    o.run(400)
    _same(sim, o, net)
    assert np.any(sim.state_field(4) != 0.0)
    sim.reset()
    sim.run(400)  # reset drops pending inputs and latched currents
    o2 = _oracle(net, cfg)
    o2.run(400)
    _same(sim, o2, net)


def test_external_input_errors():
    net, cfg = _network()
    sim = nb.Simulation(net, cfg)
    with pytest.raises(nb.NbgError, match="not an input-spike neuron"):
        sim.add_external_spikes([5], [N_IN + N_CUR])
    with pytest.raises(nb.NbgError, match="already spikes"):
        sim.add_external_spikes([5, 5], [3, 3])
    sim.add_external_spikes([7], [3])
    with pytest.raises(nb.NbgError, match="already spikes"):
        sim.add_external_spikes([7], [3])
    with pytest.raises(nb.NbgError, match="not an input-current neuron"):
        sim.add_external_currents([5], [0], [1.0])
    with pytest.raises(ValueError, match="same length"):
        sim.add_external_spikes([1, 2], [3])
    sim.run(10)
    with pytest.raises(nb.NbgError, match="in the past"):
        sim.add_external_spikes([3], [4])
    bad = Network()
    bad.add_layer(NeuronLayer.input_current(2))
    bad.add_layer(NeuronLayer("TimeDrivenLIF_Voltage_jump", 2, parameters=dict(LIF_PARAMS)))
    bad.connect(Connection(0, 2, synapse_type=0, weight=1.0, delay=1))
    with pytest.raises(nb.NbgError, match="current synapses"):
        nb.Simulation(bad, cfg)


def test_large_raster_with_external_spikes_bit_exact(oracle_lib):
    """Above 65,536 raster entries per run call the host assembles the raster
    on several threads; external spikes of recorded input neurons interleave
    with the device entries of their steps."""
    n_poi, n_in = 3000, 64
    net = Network()
    net.add_layer(NeuronLayer.input_spike(n_in, output=True))
    net.add_layer(NeuronLayer("PoissonRate", n_poi, output=True,
                              parameters={"poisson_rate_bias_hz": float32(400.0),
                                          "poisson_rate_gain_hz_per_current": float32(0.0)}))
    net.add_layer(NeuronLayer("TimeDrivenLIF_Voltage_jump", 100, output=True))
    rng = np.random.default_rng(4)
    src = rng.integers(0, n_in + n_poi, 5000).astype(np.int32)
    tgt = rng.integers(n_in + n_poi, n_in + n_poi + 100, 5000).astype(np.int32)
    net.connect(Connection(src, tgt, synapse_type=0, weight=0.3, delay=rng.integers(1, 9, 5000).astype(np.int32)))
    cfg = SimulationConfig(steps=700, timestep=0.1)
    sim = nb.Simulation(net, cfg)
    o = _oracle(net, cfg)
    pick = rng.choice(700 * n_in, 900, replace=False)
    t, i = pick // n_in, pick % n_in
    sim.add_external_spikes(t, i)
    o.add_external_spikes(t, i)
    sim.run()
    o.run(cfg.steps)
    assert len(sim.spike_raster()[0]) > 65536
    _same(sim, o, net)
