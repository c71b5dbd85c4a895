"""The oracle's external-input semantics against hand-stepped float32
trajectories (CPU).  One input-spike neuron and one input-current neuron
drive one voltage-jump LIF neuron:
  * InputSpike at step ts: recorded at ts, arrives at ts + d (V += w before
    the update at ts + d, gated by LastSpike > t_ref);
  * InputCurrent at step tc over a delay-dc current synapse: from step
    tc + dc the target's I_ext is the latched value (ProcessCurrent sets the
    total current before that step's spikes and update).
Legacy Euler update of TimeDrivenLIF_Voltage_jump.cpp:49-86."""
import numpy as np

from neuronbridge_gb300 import Connection, Network, NeuronLayer, SimulationConfig
from neuronbridge_gb300.workloads import LIF_PARAMS

f32 = np.float32


def _net():
    net = Network()
    net.add_layer(NeuronLayer.input_spike(1, output=True))
    net.add_layer(NeuronLayer.input_current(1))
    net.add_layer(NeuronLayer("TimeDrivenLIF_Voltage_jump", 1, output=True, parameters=dict(LIF_PARAMS)))
    net.connect(Connection(0, 2, synapse_type=0, weight=3.0, delay=3))
    net.connect(Connection(1, 2, synapse_type=3, weight=1.0, delay=2))
    return net, SimulationConfig(steps=10, timestep=0.1)


def _expected(steps, ts, d, tc, dc, current):
    v_rest, tau, r, dt = f32(-65.0), f32(20.0), f32(1.0), f32(0.1)
    v, i_ext, trace = f32(-65.0), f32(0.0), []
    for t in range(steps):
        if t == tc + dc:
            i_ext = f32(current)
        if t == ts + d:
            v = f32(v + f32(3.0))
        cur = f32(f32(0.0) + f32(r * i_ext) / tau)
        aux = f32(cur + f32(v_rest - v) / tau)
        v = f32(v + f32(aux * dt))
        trace.append(v)
    return np.array(trace, np.float32)


def test_input_spike_and_current_trajectory(oracle_lib):
    import oracle

    net, cfg = _net()
    o = oracle.OracleNet(net.to_native().flat(cfg.timestep))
    o.set_trace([2])
    o.add_external_spikes([2], [0])
    o.add_external_currents([1], [1], [12.5])
    o.run(10)  # 11 updates, t = 0..10
    got = o.traces().astype(np.float32).ravel()
    assert np.array_equal(got, _expected(11, ts=2, d=3, tc=1, dc=2, current=12.5))
    t, i = o.spikes()
    assert list(zip(t.tolist(), i.tolist())) == [(2, 0)]
    assert o.num_events == 1


def test_latched_currents_sum_over_current_synapses(oracle_lib):
    """Two input-current neurons into one target: each synapse keeps its last
    value, the target's current is their float sum."""
    import oracle

    net = Network()
    net.add_layer(NeuronLayer.input_current(2))
    net.add_layer(NeuronLayer("TimeDrivenLIF_Voltage_jump", 1, parameters=dict(LIF_PARAMS)))
    net.connect(Connection([0, 1], [2, 2], synapse_type=3, weight=1.0, delay=1))
    o = oracle.OracleNet(net.to_native().flat(0.1))
    o.add_external_currents([0, 2, 4], [0, 1, 0], [1.25, 0.5, -3.0])
    vals = []
    for _ in range(6):
        o.run(1)
        vals.append(float(o.state(4)[2]))
    # updates t=0,1 then one per call: I_ext after steps 0..6
    assert vals == [1.25, 1.25, 1.75, 1.75, -2.5, -2.5]
