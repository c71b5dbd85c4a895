"""Dense subnetworks through the engine: tagged networks run with the dense
runtime's semantics, bit-exact against the oracle, and the reference's
dense-subnetwork accessors (count, names, weights, snapshot, reset)."""
import numpy as np
import pytest

import neuronbridge_gb300 as nb

pytestmark = pytest.mark.gpu


def _tagged_net(seed=5):
    """Two dense subnetworks: "drive" (Poisson) feeds "core" (voltage-jump
    LIF with recurrent excitation and inhibition); one synapse group leaves
    "core" back to "drive" so that "core" has visible outputs."""
    rng = np.random.default_rng(seed)
    n_core, n_drive = 300, 200
    net = nb.Network()
    net.add_layer(nb.NeuronLayer.poisson_rate(n_drive, dense_name="drive", rate_bias_hz=400.0,
                                              rate_gain_hz_per_current=0.0))
    net.add_layer(nb.NeuronLayer("TimeDrivenLIF_Voltage_jump", n_core, parameters={"dense_subnetwork_name": "core"}))
    m = 9000
    src = np.concatenate([rng.integers(0, n_drive, m // 3), rng.integers(n_drive, n_drive + n_core, 2 * m // 3)])
    tgt = rng.integers(n_drive, n_drive + n_core, m)
    typ = (rng.random(m) < 0.2).astype(np.int32)
    net.connect(nb.Connection(src.astype(np.int32), tgt.astype(np.int32), synapse_type=typ,
                              weight=rng.uniform(0.5, 2.5, m).astype(np.float32),
                              delay=rng.integers(1, 12, m).astype(np.int32)))
    # core -> drive (Poisson rate increments: a dense -> dense connection)
    net.connect(nb.Connection(np.arange(n_drive, n_drive + 50, dtype=np.int32), np.arange(50, dtype=np.int32),
                              synapse_type=0, weight=0.1, delay=3))
    return net, nb.SimulationConfig(steps=600, timestep=0.1)


def _record_all(sim):
    for layer in range(len(sim.description.layer_count)):
        sim.lib.nbg_set_layer_record(sim._h, layer, 1)


def _raw_raster(sim):
    t, i = sim._raster_range(0, sim._num_raster())
    order = np.lexsort((i, t))
    return t[order], i[order]


def _oracle_spikes(o):
    t, i = o.spikes()
    order = np.lexsort((i, t))
    return t[order], i[order]


def test_tagged_network_runs_dense_semantics_bit_exact(oracle_lib):
    net, cfg = _tagged_net()
    sim = nb.Simulation(net, cfg)
    assert sim.semantics == "dense"
    _record_all(sim)
    sim.run()
    o = oracle_lib.OracleNet(net.to_native().flat(cfg.timestep, semantics=1))
    o.run(cfg.steps)
    ts, is_ = _raw_raster(sim)
    to, io = _oracle_spikes(o)
    assert len(ts) > 100
    assert np.array_equal(ts, to) and np.array_equal(is_, io)
    for f in range(5):
        assert np.array_equal(sim.state_field(f), o.state(f).astype(np.float32)), f
    assert sim.num_events == o.num_events


def test_dense_subnetwork_accessors():
    net, cfg = _tagged_net()
    d = net.to_native()
    sim = nb.Simulation(net, cfg)
    assert sim.dense_subnetwork_count == 2
    assert [sim.dense_subnetwork_name(k) for k in range(2)] == ["drive", "core"]
    assert sim.find_dense_subnetwork("core") == 1 and sim.find_dense_subnetwork("nope") == -1
    with pytest.raises(IndexError):
        sim.dense_subnetwork_name(2)
    with pytest.raises(KeyError):
        sim.dense_subnetwork_snapshot("nope")
    core = np.arange(200, 500)
    internal = np.flatnonzero(np.isin(d.source, core) & np.isin(d.target, core))
    assert np.array_equal(np.float32(sim.dense_subnetwork_weights(1)), d.weight[internal])
    k = int(internal[7])
    sim.set_connection_weight(k, 4.75)
    assert 4.75 in sim.dense_subnetwork_weights(1)
    sim.run(200)
    snap = sim.dense_subnetwork_snapshot("core")
    assert snap["name"] == "core" and snap["time_step"] == 200
    assert snap["local_to_original_neuron_ids"] == core.tolist()
    v = sim.state_field(0)
    assert np.array_equal(np.float32(snap["membrane_v"]), v[core])
    fired = np.flatnonzero(sim.state_field(6)[core] == 0)
    assert np.flatnonzero(np.asarray(snap["fired"])).tolist() == fired.tolist()
    assert snap["full_firing_ids"] == []
    sim.set_dense_subnetwork_full_firing_export_enabled("core")
    assert sim.dense_subnetwork_snapshot(1)["full_firing_ids"] == fired.tolist()
    # core neurons 0..49 (original 200..249) send to "drive": only they are visible outputs
    assert all(x < 50 for x in snap["visible_output_firing_ids"])


def test_reset_dense_subnetwork_matches_oracle(oracle_lib):
    net, cfg = _tagged_net(seed=9)
    sim = nb.Simulation(net, cfg)
    _record_all(sim)
    o = oracle_lib.OracleNet(net.to_native().flat(cfg.timestep, semantics=1))
    sim.run(250)
    o.run(250)
    assert sim.lib.nbg_reset_neurons(sim._h, -1, 5) != 0  # range outside the network
    assert sim.lib.nbg_reset_neurons(sim._h, 490, 20) != 0
    assert sim.lib.nbg_reset_neurons(sim._h, 10, 0) == 0  # empty range: nothing to do
    sim.reset_dense_subnetwork("core")
    o.reset_neurons(200, 300)
    for f in range(5):
        assert np.array_equal(sim.state_field(f), o.state(f).astype(np.float32)), f
    sim.run(300)
    o.run(300)
    ts, is_ = _raw_raster(sim)
    to, io = _oracle_spikes(o)
    assert np.array_equal(ts, to) and np.array_equal(is_, io)
    for f in range(5):
        assert np.array_equal(sim.state_field(f), o.state(f).astype(np.float32)), f
    assert sim.num_events == o.num_events
    assert sim.next_time == o.next_time == 551


def test_input_layer_driving_a_dense_subnetwork(oracle_lib):
    """Input-spike neurons stay in the main network (the reference's rule)
    and drive a dense-tagged LIF layer: dense semantics chosen automatically,
    external spikes delivered bit-exact against the oracle."""
    rng = np.random.default_rng(21)
    n_in, n = 32, 200
    net = nb.Network()
    net.add_layer(nb.NeuronLayer.input_spike(n_in))
    net.add_layer(nb.NeuronLayer("TimeDrivenLIF_Voltage_jump", n, parameters={"dense_subnetwork_name": "core"}))
    src = rng.integers(0, n_in, 3000).astype(np.int32)
    tgt = rng.integers(n_in, n_in + n, 3000).astype(np.int32)
    net.connect(nb.Connection(src, tgt, synapse_type=0, weight=rng.uniform(2.0, 6.0, 3000).astype(np.float32),
                              delay=rng.integers(1, 6, 3000).astype(np.int32)))
    rec_s = rng.integers(n_in, n_in + n, 2000).astype(np.int32)
    rec_t = rng.integers(n_in, n_in + n, 2000).astype(np.int32)
    net.connect(nb.Connection(rec_s, rec_t, synapse_type=(rng.random(2000) < 0.3).astype(np.int32), weight=1.5,
                              delay=rng.integers(2, 9, 2000).astype(np.int32)))
    cfg = nb.SimulationConfig(steps=400, timestep=0.1)
    sim = nb.Simulation(net, cfg)
    assert sim.semantics == "dense" and sim.dense_subnetwork_count == 1
    _record_all(sim)
    o = oracle_lib.OracleNet(net.to_native().flat(cfg.timestep, semantics=1))
    pick = rng.choice(400 * n_in, 1500, replace=False)
    t, i = pick // n_in, pick % n_in
    sim.add_external_spikes(t, i)
    o.add_external_spikes(t, i)
    sim.run()
    o.run(cfg.steps)
    ts, is_ = _raw_raster(sim)
    to, io = _oracle_spikes(o)
    assert np.array_equal(ts, to) and np.array_equal(is_, io)
    assert (is_ >= n_in).sum() > 0  # the dense layer fires
    for f in range(5):
        assert np.array_equal(sim.state_field(f), o.state(f).astype(np.float32)), f
    assert sim.num_events == o.num_events
