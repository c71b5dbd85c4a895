"""Dense-subnetwork tagging on the host: grouping, the reference's build-time
rules for dense layers, semantics selection, and the oracle's reset of one
subnetwork's neurons (no GPU)."""
import numpy as np
import pytest

import neuronbridge_gb300 as nb
from neuronbridge_gb300.simulation import _auto_semantics, _dense_groups


def _lif(count, dense=None, **kw):
    params = {} if dense is None else {"dense_subnetwork_name": dense}
    return nb.NeuronLayer("TimeDrivenLIF_Voltage_jump", count, parameters=params, **kw)


def _net(layers):
    net = nb.Network()
    for layer in layers:
        net.add_layer(layer)
    return net.to_native()


def test_groups_in_order_of_first_appearance():
    d = _net([_lif(3, "b"), _lif(2), _lif(4, "a"), _lif(1, "b")])
    assert d.layer_dense == ["b", None, "a", "b"]
    assert _dense_groups(d) == [("b", [0, 3]), ("a", [2])]


def test_dense_layer_rules_match_the_reference_build():
    with pytest.raises(RuntimeError, match="cannot be placed inside dense subnetwork"):
        _net([nb.NeuronLayer("InputSpikeNeuronModel", 2, parameters={"dense_subnetwork_name": "x"})])
    with pytest.raises(RuntimeError, match="cannot be marked isOutput=true"):
        _net([nb.NeuronLayer("TimeDrivenLIF_Voltage_jump", 2, output=True,
                             parameters={"dense_subnetwork_name": "x"})])
    with pytest.raises(RuntimeError, match="is not supported by dense GPU subnetwork"):
        _net([nb.NeuronLayer("IzhikevichCurrentRK4", 2, parameters={"dense_subnetwork_name": "x"})])
    # typed wrapper and empty name (= main network)
    d = _net([nb.NeuronLayer("PoissonRate", 2, parameters={"dense_subnetwork_name": ""}),
              nb.NeuronLayer.poisson_rate(2, dense_name="p")])
    assert d.layer_dense == [None, "p"]


def test_semantics_follow_the_tags():
    assert _auto_semantics(_net([_lif(2), _lif(3)])) == "legacy_cpu"
    assert _auto_semantics(_net([_lif(2, "a"), _lif(3, "b")])) == "dense"
    # input layers stay in the main network beside a fully dense network
    assert _auto_semantics(_net([nb.NeuronLayer("InputSpikeNeuronModel", 2), _lif(3, "a")])) == "dense"
    with pytest.raises(ValueError, match="interface routing"):
        _auto_semantics(_net([_lif(2, "a"), _lif(3)]))


def _ring_net():
    """Two dense LIF groups; group "src" fires from a strong bias, group
    "dst" receives through long delays, so arrivals are in flight at any
    step."""
    rng = np.random.default_rng(3)
    net = nb.Network()
    net.add_layer(nb.NeuronLayer("TimeDrivenLIF_Voltage_jump", 40,
                                 parameters={"dense_subnetwork_name": "src", "I_ext": nb.float32(30.0)}))
    net.add_layer(nb.NeuronLayer("TimeDrivenLIF_Voltage_jump", 30, parameters={"dense_subnetwork_name": "dst"}))
    src = rng.integers(0, 40, 600).astype(np.int32)
    tgt = rng.integers(40, 70, 600).astype(np.int32)
    net.connect(nb.Connection(src, tgt, synapse_type=0, weight=rng.uniform(1.0, 3.0, 600).astype(np.float32),
                              delay=rng.integers(5, 30, 600).astype(np.int32)))
    return net, nb.SimulationConfig(steps=200, timestep=0.1)


def test_oracle_reset_neurons_restores_initial_state_and_drops_arrivals(oracle_lib):
    net, cfg = _ring_net()
    flat = net.to_native().flat(cfg.timestep, semantics=1)
    fresh = oracle_lib.OracleNet(flat)
    a = oracle_lib.OracleNet(flat)
    a.run(120)
    assert a.num_events > 0
    a.reset_neurons(40, 30)
    for f in range(5):
        assert np.array_equal(a.state(f)[40:], fresh.state(f)[40:]), f
    # nothing already in flight reaches the reset neurons: delays are >= 5,
    # so every arrival of the next three steps was in flight at the reset
    b = oracle_lib.OracleNet(flat)
    b.run(120)
    ev_b, ev_a = b.num_events, a.num_events
    b.run(3)
    a.run(3)
    assert b.num_events > ev_b
    assert a.num_events == ev_a
    assert np.array_equal(a.state(0)[:40], b.state(0)[:40])  # the other group is untouched
