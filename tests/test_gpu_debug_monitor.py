"""DebugMonitor CSV output (the reference's DebugMonitorWriter layout) from
the GPU engine, checked against the oracle: spike rows of the watched
neurons (their layer need not be an output), state rows at the end of each
run call, sampling and flushing, weights, and that the output raster is
unchanged by the extra recording."""
import csv
import json

import numpy as np
import pytest

import neuronbridge_gb300 as nb
from neuronbridge_gb300 import Connection, Network, NeuronLayer, SimulationConfig
from neuronbridge_gb300.workloads import LIF_PARAMS

pytestmark = pytest.mark.gpu


def _network(monitored=True):
    rng = np.random.default_rng(3)
    net = Network()
    net.add_layer(NeuronLayer("TimeDrivenLIF_Voltage_jump", 40, monitored=monitored, parameters=dict(LIF_PARAMS)))
    net.add_layer(NeuronLayer("TimeDrivenLIF_Voltage_jump", 40, output=True, parameters=dict(LIF_PARAMS)))
    net.add_layer(NeuronLayer.poisson_rate(40, rate_bias_hz=7000.0, rate_gain_hz_per_current=0.0))
    ids = np.arange(40)
    net.connect(Connection((80 + ids).astype(np.int32), ids.astype(np.int32), weight=0.6, delay=1))
    src = rng.integers(0, 40, 400)
    net.connect(Connection(src.astype(np.int32), (40 + rng.integers(0, 40, 400)).astype(np.int32), weight=1.5,
                           delay=2))
    return net, SimulationConfig(steps=150, timestep=0.1)


def _rows(path):
    with open(path, newline="") as f:
        return list(csv.DictReader(f))


def _oracle(net, cfg):
    import oracle

    return oracle.OracleNet(net.to_native().flat(cfg.timestep))


def test_spikes_and_states_every_run_call(tmp_path, oracle_lib):
    net, cfg = _network()
    sim = nb.Simulation(net, cfg)
    sim.enable_debug_monitor(nb.DebugMonitorConfig(output_dir=tmp_path / "mon", record_weights=True))
    o = _oracle(net, cfg)
    frames = []
    for _ in range(3):
        sim.run(50)
        o.run(50)
        frames.append((sim.next_time - 1, o.state(0).astype(np.float32), o.state(4).astype(np.float32)))
    sim.flush_debug_monitor()
    res = sim.result()
    assert res.meta()["record_weights"] is True
    # spikes: every spike of the monitored layer (neurons 0..39), in time order
    ot, oi = o.spikes()
    sel = oi < 40
    rows = _rows(res.table_path("spikes"))
    got = [(int(r["time_step"]), int(r["global_neuron_id"])) for r in rows]
    want = sorted(zip(ot[sel].tolist(), oi[sel].tolist()))
    assert got == want and len(got) > 0
    assert {r["component_kind"] for r in rows} == {"main_network"}
    # the output raster still holds the output layer only
    t, i = sim.spike_raster()
    keep = (oi >= 40) & (oi < 80)
    assert np.array_equal(np.sort(i), np.sort(oi[keep]))
    # states at the end of each run call: v, I_ext, LastUpdate, -1, -1
    st = _rows(res.table_path("neuron_state"))
    assert len(st) == 3 * 40 * 5
    by = {(int(r["time_step"]), int(r["global_neuron_id"]), r["field_name"]): r["value"] for r in st}
    for step, v, iext in frames:
        for j in (0, 17, 39):
            assert float(by[(step, j, "v")]) == pytest.approx(float(v[j]), rel=1e-5, abs=1e-4)
            assert by[(step, j, "v")] == "%g" % v[j]
            assert float(by[(step, j, "state_1")]) == float(iext[j])
            assert by[(step, j, "state_2")] == "%g" % step
            assert by[(step, j, "state_3")] == by[(step, j, "state_4")] == "-1"
    w = _rows(res.table_path("weights"))
    assert len(w) == 3 * 440 and w[0]["synapse_id"] == "0"
    assert set(res.file_sizes()) == set(nb.DebugMonitorResult.KNOWN_TABLES)


def test_sampling_interval_and_pending_spikes(tmp_path, oracle_lib):
    net, cfg = _network()
    sim = nb.Simulation(net, cfg)
    sim.enable_debug_monitor(nb.DebugMonitorConfig(output_dir=tmp_path / "m", sample_interval_steps=100))
    o = _oracle(net, cfg)
    for _ in range(2):
        sim.run(50)  # frames would be at steps 50 and 100: only 100 is sampled
    o.run(100)
    res = sim.result()
    st = _rows(res.table_path("neuron_state"))
    assert {int(r["time_step"]) for r in st} == {100}
    n_at_100 = len(_rows(res.table_path("spikes")))
    sim.run(49)
    o.run(49)
    sim.disable_debug_monitor()  # closes: pending spikes of steps 101..149 are written
    ot, oi = o.spikes()
    assert len(_rows(tmp_path / "m" / "spikes.csv")) == int(np.sum(oi < 40)) > n_at_100
    # without a monitor the raster is the output layer's again
    sim.run(10)
    t, i = sim.spike_raster()
    assert np.all((i >= 40) & (i < 80))


def test_selection_by_ids_and_all(tmp_path):
    net, cfg = _network(monitored=False)
    sim = nb.Simulation(net, cfg)
    sim.enable_debug_monitor(nb.DebugMonitorConfig(output_dir=tmp_path / "ids", neuron_ids=[3, 45, 100]))
    sim.run(20)
    sim.flush_debug_monitor()
    st = _rows(tmp_path / "ids" / "neuron_state.csv")
    assert {int(r["global_neuron_id"]) for r in st} == {3, 45, 100}
    poisson = [r for r in st if r["global_neuron_id"] == "100"]
    assert [r["field_name"] for r in poisson] == ["v", "state_1", "state_2", "state_3", "state_4"]
    meta = json.loads((tmp_path / "ids" / "meta.json").read_text())
    assert meta["sample_interval_steps"] == 1 and meta["record_state"] is True
