"""Host union of independent networks (the host form of nbg_create_batch)."""
import ctypes

import numpy as np
import pytest

import neuronbridge_gb300 as nb
from neuronbridge_gb300 import NetworkDescription, _lib, workloads


def _plastic_net(n, seed, tau):
    rng = np.random.default_rng(seed)
    net = nb.Network()
    net.add_layer(nb.NeuronLayer("TimeDrivenLIF_Voltage_jump", n, output=True))
    net.add_layer(nb.NeuronLayer.poisson_rate(n, rate_bias_hz=3000.0, rate_gain_hz_per_current=0.0))
    net.add_learning_rule(nb.LearningRule("STDP", {"Max_LTP": nb.float32(0.01), "LTP_tau": nb.float32(tau),
                                                   "Max_LTD": nb.float32(0.012), "LTD_tau": nb.float32(tau)}))
    m = 6 * n
    src = rng.integers(0, 2 * n, m).astype(np.int32)
    tgt = rng.integers(0, n, m).astype(np.int32)
    net.connect(nb.Connection(src, tgt, synapse_type=(rng.random(m) < 0.2).astype(np.int32),
                              weight=rng.uniform(0.5, 2.0, m).astype(np.float32), max_weight=4.0,
                              delay=rng.integers(1, 8, m).astype(np.int32), synapse_rule=0))
    return net.to_native()


def test_concat_offsets_ids_and_rules():
    parts = [_plastic_net(30, 1, 15.0), _plastic_net(50, 2, 25.0), _plastic_net(20, 3, 35.0)]
    u, first, conn_first = NetworkDescription.concat(parts)
    assert first.tolist() == [0, 60, 160, 200] and u.neuron_count == 200
    assert conn_first.tolist() == [0, 180, 480, 600]
    assert u.rule_params.shape == (3, 4)
    for k, p in enumerate(parts):
        sl = slice(conn_first[k], conn_first[k + 1])
        assert np.array_equal(u.source[sl], p.source + first[k])
        assert np.array_equal(u.target[sl], p.target + first[k])
        assert np.array_equal(u.weight[sl], p.weight)
        assert np.all(u.rule[sl] == k)
        assert np.array_equal(u.rule_params[k], p.rule_params[0])
    assert len(u.layer_count) == 6 and len(u.layer_dense) == 6


def test_concat_of_batched_instances_is_the_batched_union():
    singles, union, _ = workloads.batched_lif(instances=6, lo=100, hi=900)
    u, first, _ = NetworkDescription.concat(singles)
    for key in ("layer_model", "layer_count", "layer_fparams", "layer_iparams", "source", "target", "type",
                "weight", "delay", "rule"):
        assert np.array_equal(getattr(u, key), getattr(union, key)), key


def test_batch_rejects_empty():
    with pytest.raises(ValueError):
        NetworkDescription.concat([])


def test_batch_rejects_ids_outside_their_instance():
    """Validation happens before any CUDA call, so this runs without a GPU."""
    lib = _lib.load()
    from neuronbridge_gb300.simulation import make_desc

    a = _plastic_net(40, 1, 20.0)
    b = _plastic_net(40, 2, 20.0)
    a.target = a.target.copy()
    a.target[3] = 85  # inside the union's range (160 neurons), outside instance 0 (80)
    made = [make_desc(p.flat(0.1)) for p in (a, b)]
    ptrs = (ctypes.POINTER(_lib.NetDesc) * 2)(*[ctypes.pointer(m[0]) for m in made])
    opt = _lib.Options()
    lib.nbg_default_options(ctypes.byref(opt))
    h = ctypes.c_void_p()
    st = lib.nbg_create_batch(ptrs, 2, ctypes.byref(opt), ctypes.byref(h), None)
    assert st != 0 and b"instance 0" in lib.nbg_last_error()


def test_batch_rejects_instances_with_different_timesteps():
    """Checked before any CUDA call."""
    lib = _lib.load()
    from neuronbridge_gb300.simulation import make_desc

    a = _plastic_net(40, 1, 20.0)
    made = [make_desc(a.flat(0.1)), make_desc(a.flat(0.2))]
    ptrs = (ctypes.POINTER(_lib.NetDesc) * 2)(*[ctypes.pointer(m[0]) for m in made])
    opt = _lib.Options()
    lib.nbg_default_options(ctypes.byref(opt))
    h = ctypes.c_void_p()
    assert lib.nbg_create_batch(ptrs, 2, ctypes.byref(opt), ctypes.byref(h), None) != 0
    assert b"share dt_ms" in lib.nbg_last_error()


def test_batch_rejects_an_empty_list():
    with pytest.raises(TypeError):
        nb.Simulation.batch([], nb.SimulationConfig(steps=10, timestep=0.1))
