"""Dense all-to-all delivery (split-precision tensor-core GEMM on tcgen05 and
on the legacy mma.sync path, and the FP32 CUDA-core path) against the CPU
oracle and an FP64 product.

Tolerances: the FP32 path is bit-exact (same ascending-i sequential sum as the
oracle).  The split BF16 path (W = W_hi + W_lo, binary S exact in BF16, FP32
accumulation) must stay within 2e-5 absolute of the FP64 product S W for
|W| ~ N(0, 1/N) weights; its residual representation error is about 2^-16
relative per weight, the rest is FP32 accumulation order.
"""
import numpy as np
import pytest

from neuronbridge_gb300 import NeuronLayer
from neuronbridge_gb300.dense import DensePopulations, dense_weights
from neuronbridge_gb300.workloads import LIF_PARAMS

pytestmark = pytest.mark.gpu

SPLIT_ABS_TOL = 2e-5


def _layer():
    return NeuronLayer("TimeDrivenLIF_Voltage_jump", 1, parameters=dict(LIF_PARAMS))


def _sequential_f32(w, s):
    out = np.zeros((s.shape[0], w.shape[1]), np.float32)
    for b in range(s.shape[0]):
        rows = w[np.nonzero(s[b])[0]]
        if len(rows):
            out[b] = np.cumsum(rows, axis=0, dtype=np.float32)[-1]
    return out


@pytest.mark.parametrize("precision", ["split_bf16", "split_bf16_sync"])
@pytest.mark.parametrize("n", [1024, 2048])
def test_split_bf16_delivery_error_vs_fp64(n, precision):
    w = dense_weights(n, seed=4)
    rng = np.random.default_rng(7)
    s = (rng.random((64, n)) < 0.03).astype(np.uint8)
    eng = DensePopulations(w, _layer(), precision=precision)
    got = eng.deliver(s)
    ref = s.astype(np.float64) @ w.astype(np.float64)
    err = np.abs(got.astype(np.float64) - ref)
    assert err.max() < SPLIT_ABS_TOL, err.max()
    # deterministic: the same S gives the same bits
    assert np.array_equal(got, eng.deliver(s))


def test_fp32_delivery_is_the_sequential_float_sum():
    n = 1024
    w = dense_weights(n, seed=4)
    s = (np.random.default_rng(8).random((64, n)) < 0.03).astype(np.uint8)
    eng = DensePopulations(w, _layer(), precision="fp32")
    assert np.array_equal(eng.deliver(s), _sequential_f32(w, s))


def test_fp32_simulation_bit_exact_vs_oracle(oracle_lib):
    import oracle

    n, steps = 1024, 300
    w = dense_weights(n, seed=4)
    layer = _layer()
    mid, f, ip = layer.native_params()
    eng = DensePopulations(w, layer, precision="fp32", drive_rate_hz=8000.0, drive_weight=0.5, dt=0.1)
    eng.run(steps)
    ref = oracle.OracleDense(64, n, w, f, ip, 8000.0, 0.5, 0.1)
    ref.run(steps)
    assert np.array_equal(eng.spike_counts(), ref.counts())
    assert eng.spike_counts().sum() > 0
    v, last = eng.state()
    rv, rlast, rs = ref.state()
    assert np.array_equal(v.ravel(), rv.astype(np.float32))
    assert np.array_equal(last.ravel(), rlast)
    assert np.array_equal(eng.spikes().ravel(), rs)


def test_tcgen05_and_mma_sync_paths_agree():
    n = 2048
    w = dense_weights(n, seed=4)
    s = (np.random.default_rng(9).random((64, n)) < 0.05).astype(np.uint8)
    a = DensePopulations(w, _layer(), precision="split_bf16").deliver(s)
    b = DensePopulations(w, _layer(), precision="split_bf16_sync").deliver(s)
    assert np.abs(a - b).max() < SPLIT_ABS_TOL


@pytest.mark.parametrize("precision", ["split_bf16", "split_bf16_sync"])
def test_split_bf16_simulation_tracks_fp32(precision):
    n, steps = 2048, 400
    w = dense_weights(n, seed=4)
    a = DensePopulations(w, _layer(), precision=precision).run(steps)
    b = DensePopulations(w, _layer(), precision="fp32").run(steps)
    ca, cb = a.spike_counts(), b.spike_counts()
    assert len(ca) == len(cb) == steps + 1
    # identical before any threshold decision flips, close in aggregate after
    assert np.array_equal(ca[:20], cb[:20])
    assert abs(int(ca.sum()) - int(cb.sum())) <= 0.05 * cb.sum()
