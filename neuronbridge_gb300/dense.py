"""Dense all-to-all LIF populations with tensor-core spike delivery.

Wraps the C ABI in ``include/nbg_dense.h``: 64 instances of an N-neuron
voltage-jump LIF population share one dense weight matrix W (row = pre,
column = post); each step delivers I = S W either as a BF16 split-precision
tensor-core GEMM on tcgen05 (``precision="split_bf16"``), the same GEMM on
the legacy mma.sync path (``"split_bf16_sync"``), or as an exact FP32
CUDA-core gather-sum (``"fp32"``).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .model import NeuronLayer

PRECISIONS = {"split_bf16": 0, "fp32": 1, "split_bf16_sync": 2}

_SIG = {
    "nbg_dense_create": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_float),
                                        ctypes.POINTER(_lib.LayerDesc), ctypes.c_float, ctypes.c_float,
                                        ctypes.c_float, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]),
    "nbg_dense_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "nbg_dense_run": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "nbg_dense_reset": (ctypes.c_int, [ctypes.c_void_p]),
    "nbg_dense_get_state": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_float),
                                           ctypes.POINTER(ctypes.c_int32)]),
    "nbg_dense_num_steps": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64)]),
    "nbg_dense_spike_counts": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int32)]),
    "nbg_dense_get_spikes": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint8)]),
    "nbg_dense_deliver": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint8),
                                         ctypes.POINTER(ctypes.c_float)]),
    "nbg_dense_profile": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double),
                                         ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int64)]),
}


def _bind():
    lib = _lib.load()
    for name, (res, args) in _SIG.items():
        fn = getattr(lib, name)
        fn.restype, fn.argtypes = res, args
    return lib


def _p(a, ct):
    return a.ctypes.data_as(ctypes.POINTER(ct))


class DensePopulations:
    def __init__(self, w: np.ndarray, layer: NeuronLayer, *, instances: int = 64, drive_rate_hz: float = 8000.0,
                 drive_weight: float = 0.5, dt: float = 0.1, precision: str = "split_bf16", device: int = 0):
        self.lib = _bind()
        w = np.ascontiguousarray(w, np.float32)
        if w.ndim != 2 or w.shape[0] != w.shape[1]:
            raise ValueError("w must be a square neurons x neurons matrix")
        self.B, self.N = int(instances), int(w.shape[0])
        mid, f, ip = layer.native_params()
        ld = _lib.LayerDesc()
        ld.model, ld.count = mid, self.N
        for k in range(_lib.NFP):
            ld.f[k] = float(f[k])
        for k in range(_lib.NIP):
            ld.ip[k] = int(ip[k])
        h = ctypes.c_void_p()
        st = self.lib.nbg_dense_create(self.B, self.N, _p(w, ctypes.c_float), ctypes.byref(ld), float(drive_rate_hz),
                                       float(drive_weight), float(dt), PRECISIONS[precision], int(device),
                                       ctypes.byref(h))
        if st == 1:
            raise ValueError(self.lib.nbg_last_error().decode())
        _lib.check(st)
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            self.lib.nbg_dense_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def run(self, steps: int) -> "DensePopulations":
        _lib.check(self.lib.nbg_dense_run(self._h, int(steps)))
        return self

    def reset(self) -> "DensePopulations":
        _lib.check(self.lib.nbg_dense_reset(self._h))
        return self

    def state(self):
        v = np.empty(self.B * self.N, np.float32)
        last = np.empty(self.B * self.N, np.int32)
        _lib.check(self.lib.nbg_dense_get_state(self._h, _p(v, ctypes.c_float), _p(last, ctypes.c_int32)))
        return v.reshape(self.B, self.N), last.reshape(self.B, self.N)

    def spike_counts(self) -> np.ndarray:
        n = ctypes.c_int64()
        _lib.check(self.lib.nbg_dense_num_steps(self._h, ctypes.byref(n)))
        out = np.empty(n.value, np.int32)
        if n.value:
            _lib.check(self.lib.nbg_dense_spike_counts(self._h, _p(out, ctypes.c_int32)))
        return out

    def spikes(self) -> np.ndarray:
        s = np.empty(self.B * self.N, np.uint8)
        _lib.check(self.lib.nbg_dense_get_spikes(self._h, _p(s, ctypes.c_uint8)))
        return s.reshape(self.B, self.N)

    def deliver(self, s: np.ndarray) -> np.ndarray:
        s = np.ascontiguousarray(s, np.uint8)
        if s.shape != (self.B, self.N):
            raise ValueError("s must be instances x neurons")
        out = np.empty((self.B, self.N), np.float32)
        _lib.check(self.lib.nbg_dense_deliver(self._h, _p(s, ctypes.c_uint8), _p(out, ctypes.c_float)))
        return out

    def profile(self) -> dict:
        a, b = ctypes.c_double(), ctypes.c_double()
        n = ctypes.c_int64()
        _lib.check(self.lib.nbg_dense_profile(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(n)))
        return {"device_ms": a.value, "delivery_ms": b.value, "kernel_launches": n.value}


def dense_weights(n: int = 8192, seed: int = 4) -> np.ndarray:
    """W ~ N(0, 1/n), FP32, seeded (numpy PCG64 normal draws in FP64, rounded)."""
    rng = np.random.default_rng(seed)
    return (rng.standard_normal((n, n)) / np.sqrt(n)).astype(np.float32)
