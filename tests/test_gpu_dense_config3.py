"""Dense split-precision delivery at its configuration size: 64 instances x
8,192 LIF neurons sharing one 8192 x 8192 FP32 W ~ N(0, 1/8192), 5,000 steps
(5,001 updates), through the product path (tcgen05 split-BF16 GEMM with the
LIF update fused into the same launch, ``precision="split_bf16"``), against
the FP32 CUDA-core path and the CPU oracle in FP32 and FP64.

Bounds asserted (measured on a GB300 in brackets):
* the FP32 CUDA-core path equals the FP32 oracle bit for bit over all 5,001
  updates: per-step spike counts, final V and LastSpike;
* split-BF16 delivery of the run's own spike matrices (one every 500 steps)
  is within SPLIT_ABS_TOL = 2e-5 absolute of FP64 S W [<= 1.7e-6], the FP32
  path within 1e-6 [<= 4.3e-7];
* stepping the split and FP32 paths (and the FP64 oracle) one update at a
  time, V agrees element-wise within V_TOL = 1e-4 mV at every update before
  the first update whose spike matrix differs [1.9e-5 against FP32, 2.6e-5
  against FP64], and that first difference comes no earlier than update 10
  [41 and 34];
* after it the trajectories part (the network is chaotic), and the total
  spike counts of the 5,001 updates agree within 1e-4 relative [41,317,684
  split, 41,316,957 FP32, 41,316,548 FP64]."""
import os

import numpy as np
import pytest

from neuronbridge_gb300 import NeuronLayer
from neuronbridge_gb300.dense import DensePopulations, dense_weights
from neuronbridge_gb300.workloads import LIF_PARAMS

pytestmark = pytest.mark.gpu

N, STEPS, STEPWISE = 8192, 5000, 300
SPLIT_ABS_TOL = 2e-5
FP32_ABS_TOL = 1e-6
V_TOL = 1e-4
COUNT_REL_TOL = 1e-4


@pytest.fixture(scope="module")
def run(oracle_lib):
    import torch

    import oracle

    w = dense_weights(N, seed=4)
    layer = NeuronLayer("TimeDrivenLIF_Voltage_jump", 1, parameters=dict(LIF_PARAMS))
    _, f, ip = layer.native_params()
    threads = os.cpu_count() or 1
    sp = DensePopulations(w, layer, precision="split_bf16")
    fp = DensePopulations(w, layer, precision="fp32")
    o64 = oracle.OracleDense(64, N, w, f, ip, 8000.0, 0.5, 0.1, precision=64).set_threads(threads)
    res = {"first_flip_fp32": None, "first_flip_fp64": None, "vdiff_fp32": 0.0, "vdiff_fp64": 0.0}
    # one update per call (the first call makes two) until both differences show
    for k in range(STEPWISE):
        sp.run(1)
        fp.run(1)
        o64.run(1)
        vs, vf, (v64, _, s64) = sp.state()[0].astype(np.float64), fp.state()[0], o64.state()
        ss, sf = sp.spikes(), fp.spikes()
        if res["first_flip_fp32"] is None:
            if not np.array_equal(ss, sf):
                res["first_flip_fp32"] = k + 1
            else:
                res["vdiff_fp32"] = max(res["vdiff_fp32"], float(np.abs(vs - vf).max()))
        if res["first_flip_fp64"] is None:
            if not np.array_equal(ss.ravel(), s64):
                res["first_flip_fp64"] = k + 1
            else:
                res["vdiff_fp64"] = max(res["vdiff_fp64"], float(np.abs(vs.ravel() - v64).max()))
    # the rest of the 5,000 steps, sampling the delivery error on the run's spikes
    w64 = torch.from_numpy(w).double().cuda()
    res["split_err"], res["fp32_err"] = [], []
    rest = STEPS + 1 - (STEPWISE + 1)
    while rest > 0:
        c = min(500, rest)
        sp.run(c)
        fp.run(c)
        rest -= c
        s = sp.spikes()
        ref = (torch.from_numpy(s).double().cuda() @ w64).cpu().numpy()
        res["split_err"].append(float(np.abs(sp.deliver(s) - ref).max()))
        res["fp32_err"].append(float(np.abs(fp.deliver(s) - ref).max()))
    o64.run(STEPS + 1 - (STEPWISE + 1))
    res["counts_split"], res["counts_fp32"], res["counts_fp64"] = sp.spike_counts(), fp.spike_counts(), o64.counts()
    o32 = oracle.OracleDense(64, N, w, f, ip, 8000.0, 0.5, 0.1, precision=32).set_threads(threads)
    o32.run(STEPS)
    res["counts_o32"] = o32.counts()
    v, last = fp.state()
    rv, rlast, _ = o32.state()
    res["fp32_state_equal"] = bool(np.array_equal(v.ravel(), rv.astype(np.float32)) and np.array_equal(last.ravel(),
                                                                                                      rlast))
    return res


def test_config3_fp32_path_bit_exact_vs_oracle(run):
    assert len(run["counts_fp32"]) == STEPS + 1
    assert np.array_equal(run["counts_fp32"], run["counts_o32"])
    assert run["fp32_state_equal"]


def test_config3_delivery_error_on_run_spikes(run):
    assert len(run["split_err"]) == 10
    assert max(run["split_err"]) <= SPLIT_ABS_TOL, run["split_err"]
    assert max(run["fp32_err"]) <= FP32_ABS_TOL, run["fp32_err"]


def test_config3_split_tracks_fp32_and_fp64(run):
    for ref in ("fp32", "fp64"):
        flip = run[f"first_flip_{ref}"]
        assert flip is not None and flip >= 10, (ref, flip)
        assert run[f"vdiff_{ref}"] <= V_TOL, (ref, run[f"vdiff_{ref}"])
        a, b = int(run["counts_split"].sum()), int(run[f"counts_{ref}"].sum())
        assert a > 0 and abs(a - b) <= COUNT_REL_TOL * b, (ref, a, b)
