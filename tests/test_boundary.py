"""C-ABI library and host-side mirror of the reference API (no GPU needed)."""
import ctypes

import numpy as np
import pytest

import neuronbridge_gb300 as nb
from neuronbridge_gb300 import _lib, workloads
from neuronbridge_gb300.simulation import make_desc


def test_library_exports_every_declared_symbol(nbg_lib):
    names = _lib.declared_symbols()
    assert "nbg_create" in names and "nbg_run" in names
    for name in names:
        assert hasattr(nbg_lib, name), name


def test_version_string(nbg_lib):
    assert b"sm_103a" in nbg_lib.nbg_version()


def _create(flat):
    lib = nb.load()
    desc, keep = make_desc(flat)
    h = ctypes.c_void_p()
    st = lib.nbg_create(ctypes.byref(desc), None, ctypes.byref(h))
    return st, lib.nbg_last_error().decode()


def test_create_rejects_bad_connections_before_touching_cuda(nbg_lib):
    net, _ = workloads.plain_lif(n=20, steps=10)
    flat = net.to_native().flat(0.1)
    for key, bad, msg in (("target", 10_000, "out of range"), ("delay", 0, "delay"), ("type", 3, "type"),
                          ("rule", 4, "rule")):
        f = dict(flat)
        arr = f[key].copy()
        arr[0] = bad
        f[key] = arr
        st, err = _create(f)
        assert st != 0 and msg in err, (key, st, err)


def test_create_rejects_bad_layers(nbg_lib):
    net, _ = workloads.plain_lif(n=20, steps=10)
    f = net.to_native().flat(0.1)
    f["dt"] = 0.0
    st, err = _create(f)
    assert st == 1 and "timestep" in err


def test_null_engine_calls_fail_cleanly(nbg_lib):
    assert nbg_lib.nbg_run(None, 5) == 1
    assert "null" in nbg_lib.nbg_last_error().decode()


def test_mirror_api_validation_matches_reference():
    with pytest.raises(ValueError):
        nb.NeuronLayer("PoissonRate", 0)
    with pytest.raises(ValueError):
        nb.SimulationConfig(steps=0, timestep=0.1)
    with pytest.raises(ValueError):
        nb.SimulationConfig(steps=10, timestep=0.1, event_queue="fifo")
    with pytest.raises(ValueError):
        nb.Connection([0, 1], [0, 1, 2]).normalized()
    with pytest.raises(TypeError):
        nb.Network().add_layer("not a layer")
    layer = nb.NeuronLayer("NoSuchModel", 3)
    with pytest.raises(ValueError, match="not supported"):
        layer.native_params()
    with pytest.raises(ValueError, match="random_sigma"):
        nb.NeuronLayer("TimeDrivenLIF_Voltage_jump", 3, parameters={"random_sigma": [1.0, 0.0]}).native_params()


def test_catalog_aliases_resolve_like_reference():
    assert nb.resolve_model("TimeDrivenLIF_Voltage_jump_GPU") == _lib.MODEL_LIF_VJ
    assert nb.resolve_model("TimeDrivenIzhikevic_I_Exponential_Decay") == _lib.MODEL_IZH_COND
    assert nb.resolve_model("PoissonRate_GPU") == _lib.MODEL_POISSON


def test_connection_broadcast_and_max_weight_default():
    c = nb.Connection(0, [1, 2, 3], weight=0.5).normalized()
    assert c["source"].tolist() == [0, 0, 0]
    assert c["max_weight"].tolist() == [0.5, 0.5, 0.5]
    assert c["synapse_rule"].tolist() == [-1, -1, -1]


def test_layer_defaults_follow_reference_headers():
    mid, f, ip = nb.NeuronLayer("TimeDrivenLIF_Voltage_jump", 1).native_params()
    assert (f[0], f[1], f[2], f[3], f[4], ip[0]) == (0.0, 10.0, 20.0, 1.0, -5.0, 50)
    mid, f, ip = nb.NeuronLayer("TimeDrivenIzhikevic_Exponential_Decay", 1).native_params()
    assert np.allclose(f[:6], [0.02, 0.2, -65.0, 8.0, -65.0, 30.0])
    p = nb.LearningRule("STDP").native_params()
    assert np.allclose(p, [0.92, 16.8, 0.53, 33.1])


def test_workloads_are_seeded_and_shaped():
    a, _ = workloads.plain_lif()
    b, _ = workloads.plain_lif()
    da, db = a.to_native(), b.to_native()
    assert np.array_equal(da.source, db.source) and np.array_equal(da.target, db.target)
    assert da.neuron_count == 2000
    assert 95_000 < len(da.source) < 105_000
    net, _ = workloads.izhikevich_stdp(n=1000)
    d = net.to_native()
    assert len(d.source) == 100_000
    assert np.all(np.bincount(d.target, minlength=1000) == 100)
    assert np.all(d.source != d.target)
    assert set(np.unique(d.delay)) <= set(range(10, 201, 10))
    assert np.all((d.rule == 0) == (d.source < 800))
