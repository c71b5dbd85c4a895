"""``Simulation``: the reference's run API over the GB300 engine.

Mirrors ``neuronbridge.Simulation`` (reference python/src/neuronbridge/
__init__.py:126-450) and ``_core.Simulation`` (python/bindings/
neuronbridge_core.cpp:152-520): ``init``, ``run`` (N+1 updates on the first
call), ``neuron_state(s)``, ``output_spikes``, ``get/set_connection_weight``,
``reset`` and ``bench_profiling_snapshot``.  Every call goes through the C ABI
of ``libnbg.so``; errors surface as ``ValueError`` for bad arguments (the
reference's ``py::value_error``) and :class:`NbgError` (a ``RuntimeError``)
otherwise.
"""
from __future__ import annotations

import ctypes
import os
import time
from pathlib import Path

import numpy as np

from . import _lib
from .model import Network, NetworkDescription, SimulationConfig

_SEMANTICS = {"legacy_cpu": _lib.SEM_LEGACY_CPU, "dense": _lib.SEM_DENSE}


def _p(a, ct):
    return a.ctypes.data_as(ctypes.POINTER(ct))


def make_desc(flat: dict):
    """Build the ``nbg_net_desc`` struct (and keep its arrays alive)."""
    n = len(flat["layer_model"])
    layers = (_lib.LayerDesc * n)()
    for i in range(n):
        layers[i].model = int(flat["layer_model"][i])
        layers[i].count = int(flat["layer_count"][i])
        for k in range(_lib.NFP):
            layers[i].f[k] = float(flat["layer_fparams"][i][k])
        for k in range(_lib.NIP):
            layers[i].ip[k] = int(flat["layer_iparams"][i][k])
        layers[i].output = int(bool(flat["layer_output"][i]))
    rp = flat["rule_params"]
    rules = (_lib.StdpDesc * max(1, len(rp)))()
    for r in range(len(rp)):
        rules[r].max_ltp, rules[r].ltp_tau, rules[r].max_ltd, rules[r].ltd_tau = (float(x) for x in rp[r])
    arrays = {k: np.ascontiguousarray(flat[k], dt) for k, dt in
              (("source", np.int32), ("target", np.int32), ("type", np.int32), ("weight", np.float32),
               ("max_weight", np.float32), ("delay", np.int32), ("rule", np.int32))}
    desc = _lib.NetDesc()
    desc.n_layers = n
    desc.layers = layers
    desc.n_conn = len(arrays["source"])
    desc.source = _p(arrays["source"], ctypes.c_int32)
    desc.target = _p(arrays["target"], ctypes.c_int32)
    desc.type = _p(arrays["type"], ctypes.c_int32)
    desc.weight = _p(arrays["weight"], ctypes.c_float)
    desc.max_weight = _p(arrays["max_weight"], ctypes.c_float)
    desc.delay = _p(arrays["delay"], ctypes.c_int32)
    desc.rule = _p(arrays["rule"], ctypes.c_int32)
    desc.n_rules = len(rp)
    desc.rules = rules
    desc.dt_ms = float(flat["dt"])
    desc.semantics = int(flat["semantics"])
    desc.seed = int(flat["seed"])
    return desc, (layers, rules, arrays)


class Simulation:
    """High-level facade over one GB300 engine instance."""

    def __init__(self, network: Network | NetworkDescription | str | os.PathLike, config: SimulationConfig, *,
                 build_options=None, device: int = 0, semantics: str = "legacy_cpu", seed: int = 0,
                 block_steps: int = 0, use_graph: bool = True, threads_per_block: int = 256,
                 spike_capacity: int = 0, event_log_capacity: int = 0, kernel_timing: bool = False):
        if not isinstance(config, SimulationConfig):
            raise TypeError("Simulation expects a neuronbridge_gb300.SimulationConfig")
        if semantics not in _SEMANTICS:
            raise ValueError(f"semantics must be one of {sorted(_SEMANTICS)}")
        build_started = time.perf_counter()
        self.config = config
        self.lib = _lib.load()
        if isinstance(network, (str, os.PathLike)):  # .nbnet file (the reference's path overload)
            from . import nbnet

            options = build_options or nbnet.StreamingBuildOptions()
            if not isinstance(options, nbnet.StreamingBuildOptions):
                raise TypeError("build_options must be a StreamingBuildOptions")
            native, self._build_stats = nbnet.load(network, options)
            self.network_file = Path(network).resolve()
        else:
            if build_options is not None:
                raise TypeError("build_options is only valid when Simulation receives an .nbnet path")
            native = network.to_native() if isinstance(network, Network) else network
            if not isinstance(native, NetworkDescription):
                raise TypeError("Simulation expects a neuronbridge_gb300.Network or an .nbnet path")
            self.network_file = None
            self._build_stats = {"mode": "in_memory", "neuron_count": native.neuron_count,
                                 "connection_count": int(len(native.source))}
        self.description = native
        self.flat = native.flat(config.timestep, _SEMANTICS[semantics], seed)
        desc, keep = make_desc(self.flat)
        opt = _lib.Options()
        self.lib.nbg_default_options(ctypes.byref(opt))
        opt.device = int(device)
        opt.block_steps = int(block_steps)
        opt.threads_per_block = int(threads_per_block)
        opt.spike_capacity = int(spike_capacity)
        opt.use_graph = int(bool(use_graph))
        opt.event_log_capacity = int(event_log_capacity)
        opt.kernel_timing = int(bool(kernel_timing))
        h = ctypes.c_void_p()
        st = self.lib.nbg_create(ctypes.byref(desc), ctypes.byref(opt), ctypes.byref(h))
        if st == 1:
            raise ValueError(self.lib.nbg_last_error().decode())
        _lib.check(st)
        self._h = h
        self._initialized = False
        self._trace_n = 0
        layer_start = np.concatenate([[0], np.cumsum(native.layer_count)])
        self._output_mask = np.zeros(native.neuron_count, bool)
        for i, out in enumerate(native.layer_output):
            if out:
                self._output_mask[layer_start[i]:layer_start[i + 1]] = True
        self._layer_of = np.repeat(np.arange(len(native.layer_count)), native.layer_count)
        self._layer_monitored = native.layer_monitored
        self._extra_recorded = False  # layers recorded for the monitor beyond the outputs
        self._monitor = None
        self._build_stats["total_build_seconds"] = time.perf_counter() - build_started

    @property
    def build_stats(self) -> dict:
        """Construction-path diagnostics (the reference's Simulation.build_stats)."""
        return dict(self._build_stats)

    # -------------------------------------------------------------- lifecycle
    def close(self) -> None:
        h = getattr(self, "_h", None)
        if h:
            self.lib.nbg_destroy(h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def initialized(self) -> bool:
        return self._initialized

    def init(self) -> "Simulation":
        self._initialized = True
        return self

    def run(self, steps: int | None = None) -> "Simulation":
        steps = self.config.steps if steps is None else int(steps)
        if steps <= 0:
            raise ValueError("Simulation.run steps must be positive")
        self.init()
        _lib.check(self.lib.nbg_run(self._h, steps))
        if self._monitor is not None:
            self._monitor.capture(self.next_time - 1)
        return self

    def reset(self) -> "Simulation":
        if self._monitor is not None:
            self._monitor.collect_spikes()
        _lib.check(self.lib.nbg_reset(self._h))
        if self._monitor is not None:
            self._monitor.read = 0
        self._initialized = False
        return self

    # --------------------------------------------------------- debug monitor
    def enable_debug_monitor(self, config) -> "Simulation":
        """Write CSV frames of state, spikes and weights at the end of every
        run call (the reference's Simulation.enable_debug_monitor)."""
        from .debug_monitor import DebugMonitor, DebugMonitorConfig

        if not isinstance(config, DebugMonitorConfig):
            raise TypeError("enable_debug_monitor expects a DebugMonitorConfig")
        if self._monitor is not None:
            self._monitor.close()
            self._monitor = None
        if config.enabled:
            self._monitor = DebugMonitor(self, config)
        self._debug_monitor_config = config
        return self

    def disable_debug_monitor(self) -> "Simulation":
        if self._monitor is not None:
            self._monitor.close()
            self._monitor = None
        return self

    def flush_debug_monitor(self) -> "Simulation":
        if self._monitor is not None:
            self._monitor.flush()
        return self

    def result(self):
        from .debug_monitor import DebugMonitorResult

        if getattr(self, "_debug_monitor_config", None) is None:
            raise RuntimeError("DebugMonitor is not enabled for this Simulation")
        return DebugMonitorResult(self._debug_monitor_config.output_dir)

    def _num_raster(self) -> int:
        n = ctypes.c_int64()
        _lib.check(self.lib.nbg_num_spikes(self._h, ctypes.byref(n)))
        return n.value

    def _raster_range(self, offset: int, count: int) -> tuple[np.ndarray, np.ndarray]:
        t = np.empty(count, np.int32)
        i = np.empty(count, np.int32)
        _lib.check(self.lib.nbg_get_spikes_from(self._h, int(offset), int(count), _p(t, ctypes.c_int32),
                                                _p(i, ctypes.c_int32)))
        return t, i

    # ------------------------------------------------------------------ state
    @property
    def neuron_count(self) -> int:
        n = ctypes.c_int()
        _lib.check(self.lib.nbg_num_neurons(self._h, ctypes.byref(n)))
        return n.value

    @property
    def next_time(self) -> int:
        t = ctypes.c_int()
        _lib.check(self.lib.nbg_next_time(self._h, ctypes.byref(t)))
        return t.value

    @property
    def block_steps(self) -> int:
        b = ctypes.c_int()
        _lib.check(self.lib.nbg_block_steps(self._h, ctypes.byref(b)))
        return b.value

    def set_launch(self, threads_per_block: int = 256, block_steps: int = 0) -> "Simulation":
        """Change the launch shape (speed only; results are independent of it)."""
        _lib.check(self.lib.nbg_set_launch(self._h, int(threads_per_block), int(block_steps)))
        return self

    def state_field(self, field: int) -> np.ndarray:
        out = np.empty(self.description.neuron_count, np.float32)
        _lib.check(self.lib.nbg_get_state(self._h, int(field), _p(out, ctypes.c_float)))
        return out

    def set_state_field(self, field: int, values) -> None:
        arr = np.ascontiguousarray(values, np.float32)
        if arr.shape != (self.description.neuron_count,):
            raise ValueError("state array must have one value per neuron")
        _lib.check(self.lib.nbg_set_state(self._h, int(field), _p(arr, ctypes.c_float)))

    def _state_table(self):
        return {f: self.state_field(f) for f in (_lib.FIELD_V, _lib.FIELD_U, _lib.FIELD_G_EXC, _lib.FIELD_G_INH,
                                                 _lib.FIELD_I_EXT, _lib.FIELD_LAST_SPIKE)}

    def _state_dict(self, tab, neuron_id: int) -> dict:
        if not 0 <= neuron_id < self.description.neuron_count:
            raise KeyError("original neuron id is not present in the main network")
        layer = int(self._layer_of[neuron_id])
        model = int(self.description.layer_model[layer])
        v, u, ge, gi, ie = (float(tab[f][neuron_id]) for f in range(5))
        if model == _lib.MODEL_LIF_VJ:
            values = [v, ie]
        elif model == _lib.MODEL_IZH_COND:
            values = [v, u, ge, gi, 0.0, ie]
        elif model == _lib.MODEL_IZH_RK4:
            values = [v, u, ie]
        else:
            values = [0.0, ie]
        start = int(np.sum(self.description.layer_count[:layer]))
        return {"original_neuron_id": neuron_id, "main_neuron_id": neuron_id, "local_neuron_id": neuron_id - start,
                "queue_index": 0, "is_output": bool(self._output_mask[neuron_id]), "state_variables": values,
                "last_update": self.next_time - 1, "last_spike": int(tab[_lib.FIELD_LAST_SPIKE][neuron_id])}

    def neuron_state(self, original_neuron_id: int) -> dict:
        return self._state_dict(self._state_table(), int(original_neuron_id))

    def neuron_states(self, original_neuron_ids) -> list[dict]:
        tab = self._state_table()
        return [self._state_dict(tab, int(i)) for i in original_neuron_ids]

    # ----------------------------------------------------------------- spikes
    def spike_raster(self) -> tuple[np.ndarray, np.ndarray]:
        """All spikes so far as (times, neuron ids), ordered by (time, id)."""
        n = ctypes.c_int64()
        _lib.check(self.lib.nbg_num_spikes(self._h, ctypes.byref(n)))
        t = np.empty(n.value, np.int32)
        i = np.empty(n.value, np.int32)
        _lib.check(self.lib.nbg_get_spikes(self._h, _p(t, ctypes.c_int32), _p(i, ctypes.c_int32), n.value))
        if self._extra_recorded:  # the monitor also records non-output layers
            keep = self._output_mask[i]
            t, i = t[keep], i[keep]
        return t, i

    def output_spikes(self) -> list[dict]:
        t, i = self.spike_raster()
        keep = self._output_mask[i] if len(i) else np.zeros(0, bool)
        return [{"time": int(a), "neuron_id": int(b)} for a, b in zip(t[keep], i[keep])]

    def clear_spikes(self) -> "Simulation":
        if self._monitor is not None:
            self._monitor.collect_spikes()
        _lib.check(self.lib.nbg_clear_spikes(self._h))
        if self._monitor is not None:
            self._monitor.read = 0
        return self

    @property
    def num_events(self) -> int:
        """Synaptic events delivered so far."""
        n = ctypes.c_int64()
        _lib.check(self.lib.nbg_num_events(self._h, ctypes.byref(n)))
        return n.value

    # ---------------------------------------------------------------- weights
    def weights(self) -> dict:
        s = len(self.description.source)
        w, a, b = (np.empty(s, np.float32) for _ in range(3))
        last = np.empty(s, np.int32)
        _lib.check(self.lib.nbg_get_weights(self._h, _p(w, ctypes.c_float), _p(a, ctypes.c_float),
                                            _p(b, ctypes.c_float), _p(last, ctypes.c_int32)))
        return {"weight": w, "apre": a, "apost": b, "last_update": last}

    def get_connection_weight(self, original_connection_index: int) -> float:
        idx = int(original_connection_index)
        if not 0 <= idx < len(self.description.source):
            raise IndexError("connection index out of range")
        return float(self.weights()["weight"][idx])

    def set_connection_weight(self, original_connection_index: int, weight: float) -> "Simulation":
        _lib.check(self.lib.nbg_set_weight(self._h, int(original_connection_index), float(weight)))
        return self

    def add_external_spikes(self, times, neuron_ids) -> "Simulation":
        """Spikes of input-spike neurons at the given steps, delivered over
        their synapses inside the device step loop (the reference's
        Simulation.add_external_spikes)."""
        t = np.ascontiguousarray(np.atleast_1d(times), np.int64)
        i = np.ascontiguousarray(np.atleast_1d(neuron_ids), np.int64)
        if t.shape != i.shape:
            raise ValueError("external spike times and neuron_ids must have the same length")
        t32, i32 = (np.ascontiguousarray(x, np.int32) for x in (t, i))
        _lib.check(self.lib.nbg_add_external_spikes(self._h, len(t32), _p(t32, ctypes.c_int32),
                                                    _p(i32, ctypes.c_int32)))
        return self

    def add_external_currents(self, times, neuron_ids, currents) -> "Simulation":
        """Currents sent by input-current neurons at the given steps over
        their current synapses (the reference's Simulation.add_external_currents)."""
        t = np.ascontiguousarray(np.atleast_1d(times), np.int32)
        i = np.ascontiguousarray(np.atleast_1d(neuron_ids), np.int32)
        c = np.ascontiguousarray(np.atleast_1d(currents), np.float32)
        if not (t.shape == i.shape == c.shape):
            raise ValueError("external current times, neuron_ids, and currents must have the same length")
        _lib.check(self.lib.nbg_add_external_currents(self._h, len(t), _p(t, ctypes.c_int32),
                                                      _p(i, ctypes.c_int32), _p(c, ctypes.c_float)))
        return self

    def set_current_at(self, times, neuron_ids, currents) -> "Simulation":
        """Set each neuron's external current at the start of the given step
        (the effect of a delay-d current connection from an input-current
        neuron in the reference: ProcessCurrent sets the total current)."""
        times, ids, vals = (list(np.atleast_1d(x)) for x in (times, neuron_ids, currents))
        if not (len(times) == len(ids) == len(vals)):
            raise ValueError("external current times, neuron_ids, and currents must have the same length")
        for t, i, v in zip(times, ids, vals):
            _lib.check(self.lib.nbg_set_current_at(self._h, int(t), int(i), float(v)))
        return self

    def save_weights(self, path) -> "Simulation":
        """Write all weights as an NPGR_WEIGHT_SNAPSHOT v1 file (the reference's
        Simulation.save_weights)."""
        from .weightio import write_snapshot

        try:
            write_snapshot(path, self.weights()["weight"], max(0, self.next_time - 1))
        except ValueError as exc:
            raise RuntimeError(f"SaveWeightToFile failed: {exc}") from None
        return self

    def load_weights(self, path) -> "Simulation":
        """Read an NPGR_WEIGHT_SNAPSHOT v1 file and replace all weights; the
        main block must have one weight per connection (all-or-nothing)."""
        from .weightio import read_snapshot

        try:
            snap = read_snapshot(path)
            w = np.ascontiguousarray(snap["main"], np.float32)
            if len(w) != len(self.description.source):
                raise ValueError("main weight block count does not match simulation network")
            if snap["dense"]:
                raise ValueError("dense weight block count does not match simulation dense subnetworks")
        except ValueError as exc:
            raise RuntimeError(f"LoadWeight failed: {exc}") from None
        _lib.check(self.lib.nbg_set_weights(self._h, _p(w, ctypes.c_float)))
        return self

    # ----------------------------------------------------------------- traces
    def set_trace(self, neuron_ids) -> "Simulation":
        ids = np.ascontiguousarray(neuron_ids, np.int32)
        _lib.check(self.lib.nbg_set_trace(self._h, len(ids), _p(ids, ctypes.c_int32)))
        self._trace_n = len(ids)
        return self

    def traces(self) -> np.ndarray:
        rows = ctypes.c_int64()
        _lib.check(self.lib.nbg_num_trace_rows(self._h, ctypes.byref(rows)))
        out = np.empty(rows.value * self._trace_n, np.float32)
        if out.size:
            _lib.check(self.lib.nbg_get_traces(self._h, _p(out, ctypes.c_float)))
        return out.reshape(rows.value, self._trace_n)

    def logged_events(self):
        n = ctypes.c_int64()
        _lib.check(self.lib.nbg_num_logged_events(self._h, ctypes.byref(n)))
        t = np.empty(n.value, np.int32)
        c = np.empty(n.value, np.int64)
        w = np.empty(n.value, np.float32)
        _lib.check(self.lib.nbg_get_logged_events(self._h, _p(t, ctypes.c_int32), _p(c, ctypes.c_int64),
                                                  _p(w, ctypes.c_float)))
        return t, c, w

    def bench_profiling_snapshot(self) -> dict:
        """Device timings of the last run call (CUDA events on the engine stream)."""
        tot, upd, prop = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        n = ctypes.c_int64()
        _lib.check(self.lib.nbg_profile(self._h, ctypes.byref(tot), ctypes.byref(upd), ctypes.byref(prop),
                                        ctypes.byref(n)))
        return {"device_ms": tot.value, "update_kernel_ms": upd.value, "propagate_kernel_ms": prop.value,
                "kernel_launches": n.value}
