"""The C ABI from a plain C host (tests/c_abi/abi_demo.c, compiled with gcc
against include/ and the in-tree library): it builds and links on any
machine; without a GPU nbg_create reports the CUDA error through
nbg_last_error; on a GPU its results equal the Python mirror's."""
import os
import shutil
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _build(tmp_path):
    from neuronbridge_gb300 import build

    build.build()
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    exe = str(tmp_path / "abi_demo")
    libdir = os.path.dirname(build.LIB)
    subprocess.run([cc, "-O2", "-std=c11", "-I", os.path.join(ROOT, "include"), os.path.join(HERE, "c_abi", "abi_demo.c"),
                    "-L", libdir, "-lnbg", f"-Wl,-rpath,{libdir}", "-o", exe], check=True)
    return exe


def _run(exe, *args):
    out = subprocess.run([exe, *map(str, args)], check=True, capture_output=True, text=True).stdout.split()
    return out


def test_c_host_builds_links_and_reports_errors(tmp_path):
    import torch

    exe = _build(tmp_path)
    out = _run(exe, 100)
    assert out[0] == "status"
    if not torch.cuda.is_available():
        assert int(out[1]) != 0 and out[3] == "error"


@pytest.mark.gpu
def test_c_host_matches_python_mirror(tmp_path):
    import neuronbridge_gb300 as nb

    exe = _build(tmp_path)
    out = _run(exe, 500)
    assert out[1] == "0" and out[2] == "0", out
    spikes, events = int(out[4]), int(out[6])
    n, fan = 200, 20
    net = nb.Network()
    net.add_layer(nb.NeuronLayer("TimeDrivenLIF_Voltage_jump", n, output=True,
                                 parameters={"V_rest": nb.float32(-65.0), "tau": nb.float32(20.0),
                                             "V_th": nb.float32(-50.0), "R": nb.float32(1.0),
                                             "V_reset": nb.float32(-65.0), "t_ref": nb.int32(20)}))
    net.add_layer(nb.NeuronLayer.poisson_rate(n, rate_bias_hz=4000.0, rate_gain_hz_per_current=0.0))
    ids = np.arange(n, dtype=np.int32)
    net.connect(nb.Connection(ids + n, ids, synapse_type=0, weight=2.0, delay=1))
    i = np.repeat(ids, fan)
    k = np.tile(np.arange(fan, dtype=np.int32), n)
    net.connect(nb.Connection(i, ((i * 7 + k * 13 + 1) % n).astype(np.int32),
                              synapse_type=(k % 5 == 0).astype(np.int32), weight=0.8, delay=5))
    sim = nb.Simulation(net, nb.SimulationConfig(steps=500, timestep=0.1))
    sim.run(500)
    t, ii = sim.spike_raster()
    assert spikes == len(t) > 0 and events == sim.num_events
    assert (int(out[8]), int(out[9])) == (int(t[0]), int(ii[0]))
