"""``.nbnet`` files (the reference's python/src/neuronbridge/nbnet.py format):
header and record layout, the checksum, the validation errors, the
parameter encoding, and bounded-memory loading into the same flat
description an in-memory Network produces."""
import hashlib
import json
import struct

import numpy as np
import pytest

from neuronbridge_gb300 import Connection, LearningRule, Network, NeuronLayer, float32, int32, nbnet
from neuronbridge_gb300.workloads import LIF_PARAMS, izhikevich_stdp


def _network():
    net = Network()
    net.add_layer(NeuronLayer("TimeDrivenLIF_Voltage_jump", 5, output=True, parameters=dict(LIF_PARAMS)))
    net.add_layer(NeuronLayer.poisson_rate(3, rate_bias_hz=800.0, rate_gain_hz_per_current=0.0))
    net.add_learning_rule(LearningRule("STDP", {"Max_LTP": float32(0.1), "LTP_tau": float32(20.0)}))
    net.connect(Connection([5, 6, 7], [0, 1, 2], weight=[0.5, 0.25, 0.125], delay=1))
    net.connect(Connection(0, [1, 2, 3, 4], synapse_type=1, weight=2.5, max_weight=4.0, delay=3, synapse_rule=0))
    return net


def test_layout_header_records_and_checksum(tmp_path):
    path = tmp_path / "net.nbnet"
    res = nbnet.from_network(_network(), path)
    raw = path.read_bytes()
    magic, major, minor, flags, rsize, msize, count, digest = struct.unpack_from("<8sHHIIQQ32s", raw)
    assert (magic, major, minor, flags, rsize, count) == (b"NBNET01\0", 1, 0, 1, 32, 7)
    hsize = struct.calcsize("<8sHHIIQQ32s")
    meta = json.loads(raw[hsize:hsize + msize])
    assert sorted(meta) == ["input_convs", "layers", "learning_rules", "outer_dynamic_connections", "outer_dynamics"]
    assert meta["layers"][0]["parameters"]["t_ref"] == {"__neuronbridge_parameter__": "int32", "value": 20}
    assert meta["layers"][1]["model"] == "PoissonRate"
    assert digest == hashlib.sha256(raw[hsize:]).digest() and res.sha256 == digest.hex()
    rec = struct.unpack_from("<IIiffIii", raw, hsize + msize + 32 * 4)  # 5th record: 0 -> 2 inhibitory plastic
    assert rec == (0, 2, 1, 2.5, 4.0, 3, 0, -1)
    assert len(raw) == hsize + msize + 7 * 32 == res.file_bytes


@pytest.mark.parametrize("mmap", [True, False])
def test_load_matches_in_memory_description(tmp_path, mmap):
    net, _ = izhikevich_stdp(n=3000, in_degree=40)
    path = tmp_path / "izh.nbnet"
    nbnet.from_network(net, path)
    a = net.to_native()
    # a 1 MiB budget makes the 120k records stream in four batches
    b, stats = nbnet.load(path, nbnet.StreamingBuildOptions(memory_budget_mb=1, mmap=mmap))
    for k in ("source", "target", "type", "weight", "max_weight", "delay", "rule", "layer_model", "layer_count",
              "layer_fparams", "layer_iparams", "layer_output", "rule_params"):
        assert np.array_equal(getattr(a, k), getattr(b, k)), k
    assert stats["batch_records"] == 32768 and stats["runtime_build_path"] == "streaming_direct"
    assert stats["connection_count"] == len(a.source)


def test_from_batches_and_builder_errors(tmp_path):
    layers = [NeuronLayer.input_spike(4), NeuronLayer("TimeDrivenLIF_Voltage_jump", 4, parameters=dict(LIF_PARAMS))]
    batches = [{"source": [0, 1], "target": [4, 5], "weight": 1.0, "delay": 2},
               {"source": np.arange(4), "target": np.arange(4, 8), "weight": np.linspace(0.1, 0.4, 4)}]
    res = nbnet.from_batches(tmp_path / "b.nbnet", layers, batches)
    assert res.connection_count == 6 and nbnet.is_valid(tmp_path / "b.nbnet")
    with pytest.raises(FileExistsError):
        nbnet.from_batches(tmp_path / "b.nbnet", layers, batches)
    with pytest.raises(ValueError, match="out of range"):
        nbnet.from_batches(tmp_path / "c.nbnet", layers, [{"source": [0], "target": [8]}])
    with pytest.raises(ValueError, match="finite"):
        nbnet.from_batches(tmp_path / "d.nbnet", layers, [{"source": [0], "target": [4], "weight": np.inf}])
    with pytest.raises(ValueError, match="length must be 1 or 2"):
        nbnet.from_batches(tmp_path / "e.nbnet", layers, [{"source": [0, 1], "target": [4, 5], "delay": [1, 2, 3]}])
    assert not list(tmp_path.glob(".*.tmp"))  # spools removed on failure


def test_validation_errors(tmp_path):
    path = tmp_path / "net.nbnet"
    nbnet.from_network(_network(), path)
    good = path.read_bytes()
    cases = {
        "invalid nbnet magic": b"XBNET01\0" + good[8:],
        "unsupported nbnet major version": good[:8] + struct.pack("<H", 2) + good[10:],
        "size mismatch": good + b"\0",
        "checksum mismatch": good[:-1] + bytes([good[-1] ^ 1]),
        "truncated nbnet header": good[:20],
    }
    for reason, data in cases.items():
        bad = tmp_path / "bad.nbnet"
        bad.write_bytes(data)
        rep = nbnet.validate(bad)
        assert not rep.valid and reason in rep.errors[0], (reason, rep.errors)
    # a flipped record bit is caught only by the checksum
    bad.write_bytes(cases["checksum mismatch"])
    assert nbnet.is_valid(bad, verify_checksum=False) and not nbnet.is_valid(bad, verify_checksum=True)
    info = nbnet.inspect(path)
    assert (info.neuron_count, info.connection_count, info.version) == (8, 7, (1, 0))


def test_unsupported_content_is_rejected(tmp_path):
    path = tmp_path / "t.nbnet"
    layers = [NeuronLayer("TimeDrivenLIF_Voltage_jump", 2, parameters=dict(LIF_PARAMS))]
    nbnet.from_batches(path, layers, [{"source": [0], "target": [1], "trigger_rule": 0}])
    with pytest.raises(ValueError, match="trigger rules"):
        nbnet.load(path)
    assert nbnet.decode_parameter(nbnet.encode_parameter({"a": int32(3), "b": 1.5, "c": [1, 2]})) == \
        {"a": int32(3), "b": 1.5, "c": [1, 2]}
