"""CPU oracle for the NeuronBridge step loop -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg may import this package, and only as the checker.  The product package
(``neuronbridge_gb300``) never imports it.

``nbg_oracle.c`` restates the reference's legacy CPU semantics (see its header
for the file:line map).  It is compiled twice by :func:`build` with gcc:
``REAL=float`` (``orc32_*``, the FP32 restatement) and ``REAL=double``
(``orc64_*``, the FP64 oracle), both with ``-ffp-contract=off`` so every float
operation rounds once, as in the reference's scalar C++.

Parity pins: ``tests/test_oracle_kat.py`` checks this oracle against the
reference's own known-answer vectors (``tests/golden/``, generated from the
reference's ``numerical_accuracy_tests.py`` by ``tests/golden/make_golden.py``).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(_HERE, "_build")
_SRC = os.path.join(_HERE, "nbg_oracle.c")
_LOCK = threading.Lock()
_LIBS: dict = {}

NFP = 16
NIP = 4


def _lib_path(prec: int) -> str:
    return os.path.join(_BUILD, f"libnbg_oracle{prec}.so")


def build(force: bool = False) -> None:
    """Compile the FP32 and FP64 oracle libraries (gcc, a few seconds)."""
    os.makedirs(_BUILD, exist_ok=True)
    jobs = []
    for prec, defs in ((32, ["-DREAL=float", "-DORC(n)=orc32_##n"]),
                       (64, ["-DREAL=double", "-DREAL_IS_DOUBLE", "-DORC(n)=orc64_##n"])):
        out = _lib_path(prec)
        if not force and os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(_SRC):
            continue
        cmd = ["gcc", "-O2", "-std=c11", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
               *defs, _SRC, "-o", out + ".tmp", "-lm"]
        jobs.append((subprocess.Popen(cmd), out))
    for proc, out in jobs:
        if proc.wait() != 0:
            raise RuntimeError("oracle build failed")
        os.replace(out + ".tmp", out)


_REF_DIR = os.path.join(_HERE, "_ref")
_REF_STDP = os.path.join(_REF_DIR, "libnbg_ref_stdp.so")


def build_ref() -> str | None:
    """Compile the reference's own pair-STDP code path (its STDP.cpp,
    STDP_State.cpp and the classes they use, from the reference tree, with
    oracle/ref_stdp/Makefile) into oracle/_ref/.  The reference tree is the
    Makefile's REF, or the NBG_REFERENCE_ROOT environment variable.  Returns
    the library path, or None when the reference tree is not on this machine
    (the recipe then has nothing to compile)."""
    cmd = ["make", "-s", "-C", os.path.join(_HERE, "ref_stdp"), "-j4"]
    root = os.environ.get("NBG_REFERENCE_ROOT")
    if root:
        cmd.append(f"REF={root}")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        if "No rule to make target" in r.stderr:
            return None
        raise RuntimeError("reference STDP build failed:\n" + r.stderr)
    return _REF_STDP


def ref_stdp_run(w0, wmax, max_ltp, ltp_tau, max_ltd, ltd_tau, dt, pre, post):
    """Replay a pre/post event schedule through the reference's own STDP
    (oracle/_ref, see build_ref).  ``pre`` is [ticks][connections] and
    ``post`` [ticks] (0/1).  Returns (weights after every tick
    [ticks][connections], Apre, Apost, LastUpdate) as float32 / int32."""
    lib = ctypes.CDLL(_REF_STDP)
    f32p, i32p, u8p = (ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_int),
                       ctypes.POINTER(ctypes.c_uint8))
    fn = lib.nbgref_stdp_run
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_int, f32p, f32p, ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                   ctypes.c_float, ctypes.c_int, u8p, u8p, f32p, f32p, f32p, i32p]
    w0 = np.ascontiguousarray(w0, np.float32)
    wmax = np.ascontiguousarray(wmax, np.float32)
    pre = np.ascontiguousarray(pre, np.uint8)
    post = np.ascontiguousarray(post, np.uint8)
    ticks, n = pre.shape
    traj = np.empty((ticks, n), np.float32)
    apre, apost = np.empty(n, np.float32), np.empty(n, np.float32)
    last = np.empty(n, np.int32)
    st = fn(n, _ptr(w0, ctypes.c_float), _ptr(wmax, ctypes.c_float), max_ltp, ltp_tau, max_ltd, ltd_tau, dt, ticks,
            _ptr(pre, ctypes.c_uint8), _ptr(post, ctypes.c_uint8), _ptr(traj, ctypes.c_float),
            _ptr(apre, ctypes.c_float), _ptr(apost, ctypes.c_float), _ptr(last, ctypes.c_int))
    if st != 0:
        raise ValueError("reference STDP driver rejected the schedule")
    return traj, apre, apost, last


def _lib(prec: int):
    with _LOCK:
        if prec in _LIBS:
            return _LIBS[prec]
        build()
        lib = ctypes.CDLL(_lib_path(prec))
        p = f"orc{prec}_"
        vp, i32p, f32p, f64p, i64p = (ctypes.c_void_p, ctypes.POINTER(ctypes.c_int),
                                      ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_double),
                                      ctypes.POINTER(ctypes.c_int64))
        sig = {
            "create": (vp, [ctypes.c_int, i32p, i32p, f32p, i32p, ctypes.c_int64, i32p, i32p, i32p, f32p, f32p,
                            i32p, i32p, ctypes.c_int, f32p, ctypes.c_float, ctypes.c_int, ctypes.c_uint64,
                            ctypes.c_char_p, ctypes.c_int]),
            "destroy": (None, [vp]),
            "run": (ctypes.c_int, [vp, ctypes.c_int]),
            "next_time": (ctypes.c_int, [vp]),
            "num_spikes": (ctypes.c_int64, [vp]),
            "num_events": (ctypes.c_int64, [vp]),
            "num_synapses": (ctypes.c_int64, [vp]),
            "get_spikes": (None, [vp, i32p, i32p]),
            "get_state": (None, [vp, ctypes.c_int, f64p]),
            "set_state": (None, [vp, ctypes.c_int, f64p]),
            "get_weights": (None, [vp, f64p, f64p, f64p, i32p]),
            "set_trace": (None, [vp, ctypes.c_int, i32p]),
            "get_traces": (ctypes.c_int64, [vp, f64p]),
            "set_event_log": (None, [vp, ctypes.c_int]),
            "num_logged_events": (ctypes.c_int64, [vp]),
            "get_events": (None, [vp, i32p, i64p, f64p]),
            "set_threads": (None, [vp, ctypes.c_int]),
            "add_current": (None, [vp, ctypes.c_int, ctypes.c_int, ctypes.c_double]),
            "add_external_spike": (None, [vp, ctypes.c_int, ctypes.c_int]),
            "set_decay_table": (None, [vp, ctypes.c_int64, f32p]),
            "reset_neurons": (None, [vp, ctypes.c_int, ctypes.c_int]),
            "add_external_current": (None, [vp, ctypes.c_int, ctypes.c_int, ctypes.c_double]),
            "dense_create": (vp, [ctypes.c_int, ctypes.c_int, f32p, f32p, i32p, ctypes.c_float, ctypes.c_float,
                                  ctypes.c_float]),
            "dense_destroy": (None, [vp]),
            "dense_run": (ctypes.c_int, [vp, ctypes.c_int]),
            "dense_set_threads": (None, [vp, ctypes.c_int]),
            "dense_num_steps": (ctypes.c_int64, [vp]),
            "dense_counts": (None, [vp, i32p]),
            "dense_state": (None, [vp, f64p, i32p, ctypes.POINTER(ctypes.c_uint8)]),
            "poisson_hash": (ctypes.c_float, [ctypes.c_int, ctypes.c_int]),
            "gauss12": (ctypes.c_double, [ctypes.c_uint64, ctypes.c_int, ctypes.c_int]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(lib, p + name)
            fn.restype = res
            fn.argtypes = args
        _LIBS[prec] = lib
        return lib


def _ptr(a, ctype):
    return a.ctypes.data_as(ctypes.POINTER(ctype))


def poisson_hash(neuron_index: int, time_step: int) -> float:
    return float(_lib(32).orc32_poisson_hash(int(neuron_index), int(time_step)))


def gauss12(seed: int, neuron: int, t: int) -> float:
    return float(_lib(32).orc32_gauss12(int(seed), int(neuron), int(t)))


class OracleNet:
    """One simulated network.  ``desc`` is the flat description produced by
    ``neuronbridge_gb300.NetworkDescription.flat()`` (plain numpy arrays)."""

    def __init__(self, desc: dict, precision: int = 32):
        self.prec = precision
        self.lib = _lib(precision)
        self._f = lambda name: getattr(self.lib, f"orc{precision}_{name}")
        d = {k: (np.ascontiguousarray(v) if isinstance(v, np.ndarray) else v) for k, v in desc.items()}
        self._keep = d
        err = ctypes.create_string_buffer(256)
        self.n_neurons = int(np.sum(d["layer_count"]))
        self.h = self._f("create")(
            int(len(d["layer_model"])), _ptr(d["layer_model"], ctypes.c_int), _ptr(d["layer_count"], ctypes.c_int),
            _ptr(d["layer_fparams"], ctypes.c_float), _ptr(d["layer_iparams"], ctypes.c_int),
            int(len(d["source"])), _ptr(d["source"], ctypes.c_int), _ptr(d["target"], ctypes.c_int),
            _ptr(d["type"], ctypes.c_int), _ptr(d["weight"], ctypes.c_float), _ptr(d["max_weight"], ctypes.c_float),
            _ptr(d["delay"], ctypes.c_int), _ptr(d["rule"], ctypes.c_int), int(len(d["rule_params"])),
            _ptr(d["rule_params"], ctypes.c_float), float(d["dt"]), int(d["semantics"]), int(d["seed"]),
            err, 256)
        if not self.h:
            raise ValueError("oracle rejected the network: " + err.value.decode())

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            self._f("destroy")(h)
            self.h = None

    def run(self, steps: int) -> "OracleNet":
        if self._f("run")(self.h, int(steps)) != 0:
            raise ValueError("steps must be positive")
        return self

    @property
    def next_time(self) -> int:
        return int(self._f("next_time")(self.h))

    @property
    def num_events(self) -> int:
        return int(self._f("num_events")(self.h))

    def spikes(self):
        n = int(self._f("num_spikes")(self.h))
        t = np.empty(n, np.int32)
        i = np.empty(n, np.int32)
        if n:
            self._f("get_spikes")(self.h, _ptr(t, ctypes.c_int), _ptr(i, ctypes.c_int))
        return t, i

    def state(self, field: int) -> np.ndarray:
        out = np.empty(self.n_neurons, np.float64)
        self._f("get_state")(self.h, int(field), _ptr(out, ctypes.c_double))
        return out

    def weights(self):
        s = int(self._f("num_synapses")(self.h))
        w = np.empty(s, np.float64)
        a = np.empty(s, np.float64)
        b = np.empty(s, np.float64)
        last = np.empty(s, np.int32)
        if s:
            self._f("get_weights")(self.h, _ptr(w, ctypes.c_double), _ptr(a, ctypes.c_double),
                                   _ptr(b, ctypes.c_double), _ptr(last, ctypes.c_int))
        return w, a, b, last

    def set_trace(self, ids) -> None:
        ids = np.ascontiguousarray(ids, np.int32)
        self._keep["trace_ids"] = ids
        self._f("set_trace")(self.h, int(len(ids)), _ptr(ids, ctypes.c_int))
        self._ntrace = len(ids)

    def traces(self) -> np.ndarray:
        n = int(self._f("get_traces")(self.h, None))
        out = np.empty(n, np.float64)
        if n:
            self._f("get_traces")(self.h, _ptr(out, ctypes.c_double))
        return out.reshape(-1, self._ntrace)

    def set_threads(self, threads: int) -> "OracleNet":
        """OpenMP threads for the per-step loops (results do not change)."""
        self._f("set_threads")(self.h, int(threads))
        return self

    def add_current(self, t: int, neuron: int, value: float) -> None:
        """Set neuron's external current to ``value`` at the start of step t."""
        self._f("add_current")(self.h, int(t), int(neuron), float(value))

    def set_decay_table(self, table) -> "OracleNet":
        """Use the given STDP decay factors ([rule][2][len] float32) instead of
        expf: the dense-runtime profile's factors come from CUDA's expf."""
        tab = np.ascontiguousarray(table, np.float32)
        self._keep["dtab"] = tab
        self._f("set_decay_table")(self.h, int(tab.shape[-1]), _ptr(tab, ctypes.c_float))
        return self

    def add_external_spikes(self, times, neurons) -> "OracleNet":
        """InputSpike events: each neuron spikes at its step."""
        for t, i in zip(np.atleast_1d(times), np.atleast_1d(neurons)):
            self._f("add_external_spike")(self.h, int(t), int(i))
        return self

    def add_external_currents(self, times, neurons, values) -> "OracleNet":
        """InputCurrent events sent over the neurons' current synapses."""
        for t, i, v in zip(np.atleast_1d(times), np.atleast_1d(neurons), np.atleast_1d(values)):
            self._f("add_external_current")(self.h, int(t), int(i), float(np.float32(v)))
        return self

    def reset_neurons(self, first: int, count: int) -> "OracleNet":
        self._f("reset_neurons")(self.h, int(first), int(count))
        return self

    def set_event_log(self, on: bool = True) -> None:
        self._f("set_event_log")(self.h, int(bool(on)))

    def events(self):
        n = int(self._f("num_logged_events")(self.h))
        t = np.empty(n, np.int32)
        c = np.empty(n, np.int64)
        w = np.empty(n, np.float64)
        if n:
            self._f("get_events")(self.h, _ptr(t, ctypes.c_int), _ptr(c, ctypes.c_int64), _ptr(w, ctypes.c_double))
        return t, c, w


class OracleDense:
    """B instances x N voltage-jump LIF neurons sharing a dense W (row = pre):
    the semantics of the GPU dense delivery engine (include/nbg_dense.h)."""

    def __init__(self, instances: int, neurons: int, w, fparams, iparams, drive_rate_hz: float,
                 drive_weight: float, dt: float, precision: int = 32):
        self.lib = _lib(precision)
        self._f = lambda name: getattr(self.lib, f"orc{precision}_{name}")
        self.B, self.N = int(instances), int(neurons)
        self.w = np.ascontiguousarray(w, np.float32)
        self.fp = np.ascontiguousarray(fparams, np.float32)
        self.ip = np.ascontiguousarray(iparams, np.int32)
        self.h = self._f("dense_create")(self.B, self.N, _ptr(self.w, ctypes.c_float), _ptr(self.fp, ctypes.c_float),
                                         _ptr(self.ip, ctypes.c_int), float(drive_rate_hz), float(drive_weight),
                                         float(dt))

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            self._f("dense_destroy")(h)
            self.h = None

    def set_threads(self, threads: int) -> "OracleDense":
        """OpenMP threads over instances (results do not change)."""
        self._f("dense_set_threads")(self.h, int(threads))
        return self

    def run(self, steps: int) -> "OracleDense":
        if self._f("dense_run")(self.h, int(steps)) != 0:
            raise ValueError("steps must be positive")
        return self

    def counts(self) -> np.ndarray:
        n = int(self._f("dense_num_steps")(self.h))
        out = np.empty(n, np.int32)
        if n:
            self._f("dense_counts")(self.h, _ptr(out, ctypes.c_int))
        return out

    def state(self):
        tot = self.B * self.N
        v = np.empty(tot, np.float64)
        last = np.empty(tot, np.int32)
        s = np.empty(tot, np.uint8)
        self._f("dense_state")(self.h, _ptr(v, ctypes.c_double), _ptr(last, ctypes.c_int),
                               s.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)))
        return v, last, s
