"""ctypes binding of the C ABI in ``include/nbg.h``.

The library is built in-tree by :mod:`neuronbridge_gb300.build`.  There is no
fallback: if the shared library is missing or fails to load, every entry point
raises, so a CPU path can never stand in for the CUDA kernels.
"""
from __future__ import annotations

import ctypes
import os
import threading

from . import build as _build

NFP = 16
NIP = 4

MODEL_LIF_VJ = 0
MODEL_IZH_COND = 1
MODEL_IZH_RK4 = 2
MODEL_POISSON = 3
MODEL_INPUT_SPIKE = 4
MODEL_INPUT_CURRENT = 5
SYN_CURRENT = 3

SEM_LEGACY_CPU = 0
SEM_DENSE = 1

FIELD_V = 0
FIELD_U = 1
FIELD_G_EXC = 2
FIELD_G_INH = 3
FIELD_I_EXT = 4
FIELD_LAST_SPIKE = 6

STATUS = {0: "OK", 1: "INVALID", 2: "CUDA", 3: "OOM", 4: "OVERFLOW", 5: "STATE", 6: "TIMEOUT", 7: "UNSUPPORTED"}


class LayerDesc(ctypes.Structure):
    _fields_ = [("model", ctypes.c_int), ("count", ctypes.c_int), ("f", ctypes.c_float * NFP),
                ("ip", ctypes.c_int * NIP), ("output", ctypes.c_int)]


class StdpDesc(ctypes.Structure):
    _fields_ = [("max_ltp", ctypes.c_float), ("ltp_tau", ctypes.c_float), ("max_ltd", ctypes.c_float),
                ("ltd_tau", ctypes.c_float)]


_i32p = ctypes.POINTER(ctypes.c_int32)
_f32p = ctypes.POINTER(ctypes.c_float)
_i64p = ctypes.POINTER(ctypes.c_int64)
_f64p = ctypes.POINTER(ctypes.c_double)


class NetDesc(ctypes.Structure):
    _fields_ = [("n_layers", ctypes.c_int), ("layers", ctypes.POINTER(LayerDesc)), ("n_conn", ctypes.c_int64),
                ("source", _i32p), ("target", _i32p), ("type", _i32p), ("weight", _f32p),
                ("max_weight", _f32p), ("delay", _i32p), ("rule", _i32p), ("n_rules", ctypes.c_int),
                ("rules", ctypes.POINTER(StdpDesc)), ("dt_ms", ctypes.c_float), ("semantics", ctypes.c_int),
                ("seed", ctypes.c_uint64)]


class Options(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("block_steps", ctypes.c_int), ("threads_per_block", ctypes.c_int),
                ("spike_capacity", ctypes.c_int64), ("use_graph", ctypes.c_int),
                ("event_log_capacity", ctypes.c_int64), ("kernel_timing", ctypes.c_int)]


class NbgError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"[{STATUS.get(status, status)}] {msg}")
        self.status = status


_LOCK = threading.Lock()
_LIB = None

_SIGNATURES = {
    "nbg_last_error": (ctypes.c_char_p, []),
    "nbg_version": (ctypes.c_char_p, []),
    "nbg_default_options": (None, [ctypes.POINTER(Options)]),
    "nbg_create": (ctypes.c_int, [ctypes.POINTER(NetDesc), ctypes.POINTER(Options), ctypes.POINTER(ctypes.c_void_p)]),
    "nbg_create_batch": (ctypes.c_int, [ctypes.POINTER(ctypes.POINTER(NetDesc)), ctypes.c_int, ctypes.POINTER(Options),
                                        ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_int64)]),
    "nbg_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "nbg_run": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "nbg_reset": (ctypes.c_int, [ctypes.c_void_p]),
    "nbg_reset_neurons": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]),
    "nbg_next_time": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int)]),
    "nbg_num_neurons": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int)]),
    "nbg_num_synapses": (ctypes.c_int, [ctypes.c_void_p, _i64p]),
    "nbg_block_steps": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int)]),
    "nbg_set_launch": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]),
    "nbg_get_state": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, _f32p]),
    "nbg_set_state": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, _f32p]),
    "nbg_num_spikes": (ctypes.c_int, [ctypes.c_void_p, _i64p]),
    "nbg_get_spikes": (ctypes.c_int, [ctypes.c_void_p, _i32p, _i32p, ctypes.c_int64]),
    "nbg_clear_spikes": (ctypes.c_int, [ctypes.c_void_p]),
    "nbg_num_events": (ctypes.c_int, [ctypes.c_void_p, _i64p]),
    "nbg_get_weights": (ctypes.c_int, [ctypes.c_void_p, _f32p, _f32p, _f32p, _i32p]),
    "nbg_set_weight": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.c_float]),
    "nbg_set_weights": (ctypes.c_int, [ctypes.c_void_p, _f32p]),
    "nbg_get_spikes_from": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, _i32p, _i32p]),
    "nbg_set_layer_record": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]),
    "nbg_get_decay_table": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int64, _f32p,
                                           ctypes.POINTER(ctypes.c_int64)]),
    "nbg_add_external_spikes": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, _i32p, _i32p]),
    "nbg_add_external_currents": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, _i32p, _i32p, _f32p]),
    "nbg_set_current_at": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_float]),
    "nbg_set_trace": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, _i32p]),
    "nbg_num_trace_rows": (ctypes.c_int, [ctypes.c_void_p, _i64p]),
    "nbg_get_traces": (ctypes.c_int, [ctypes.c_void_p, _f32p]),
    "nbg_num_logged_events": (ctypes.c_int, [ctypes.c_void_p, _i64p]),
    "nbg_get_logged_events": (ctypes.c_int, [ctypes.c_void_p, _i32p, _i64p, _f32p]),
    "nbg_profile": (ctypes.c_int, [ctypes.c_void_p, _f64p, _f64p, _f64p, _i64p]),
    "nbg_raster_profile": (ctypes.c_int, [ctypes.c_void_p, _f64p, _f64p, _f64p, _i64p]),
}


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load ``libnbg.so`` (building it first if absent) and bind the C ABI."""
    global _LIB
    with _LOCK:
        if _LIB is not None:
            return _LIB
        path = lib_path()
        if not os.path.exists(path):
            if not build_if_missing:
                raise RuntimeError(f"{path} is missing: run neuronbridge_gb300.build.build() first")
            _build.build()
        lib = ctypes.CDLL(path)
        for name, (res, args) in _SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = lib
        return lib


def check(status: int) -> None:
    if status != 0:
        raise NbgError(status, load().nbg_last_error().decode(errors="replace"))


def declared_symbols(header_dir: str | None = None) -> list[str]:
    """Names of every function declared in ``include/*.h``."""
    import re

    header_dir = header_dir or _build.INCLUDE
    names = []
    for h in sorted(os.listdir(header_dir)):
        if not h.endswith(".h"):
            continue
        text = open(os.path.join(header_dir, h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += re.findall(r"\b(nbg\w*)\s*\(", text)
    return sorted(set(names))
