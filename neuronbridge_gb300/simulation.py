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
from .model import CATALOG, Network, NetworkDescription, SimulationConfig

_SEMANTICS = {"legacy_cpu": _lib.SEM_LEGACY_CPU, "dense": _lib.SEM_DENSE}
_MODEL_NAMES = {mid: name for name, (mid, _) in CATALOG.items()}


def _dense_groups(desc: NetworkDescription) -> list[tuple[str, list[int]]]:
    """(name, layer indices) of each dense subnetwork, in order of first appearance."""
    groups: dict[str, list[int]] = {}
    for layer, name in enumerate(getattr(desc, "layer_dense", [])):
        if name:
            groups.setdefault(name, []).append(layer)
    return list(groups.items())


def _auto_semantics(desc: NetworkDescription) -> str:
    """Dense-runtime semantics when every layer with dynamics is in a dense
    subnetwork, the legacy CPU semantics when none is.  Input layers always
    belong to the main network (the reference rejects them in a subnetwork)."""
    names = getattr(desc, "layer_dense", [None] * len(desc.layer_count))
    dynamic = [i for i, m in enumerate(desc.layer_model)
               if m not in (_lib.MODEL_INPUT_SPIKE, _lib.MODEL_INPUT_CURRENT)]
    tagged = [i for i in dynamic if names[i]]
    if not tagged:
        return "legacy_cpu"
    if len(tagged) == len(dynamic):
        return "dense"
    raise ValueError("main-network layers beside dense-subnetwork layers need the reference's interface routing, "
                     "which the GB300 engine does not build: tag every layer with dynamics or none, or pass "
                     "semantics='legacy_cpu' or 'dense' to run the whole network with one semantics")


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
                 build_options=None, device: int = 0, semantics: str = "auto", seed: int = 0,
                 block_steps: int = 0, use_graph: bool = True, threads_per_block: int = 256,
                 spike_capacity: int = 0, event_log_capacity: int = 0, kernel_timing: bool = False,
                 _instances: list | None = None):
        if not isinstance(config, SimulationConfig):
            raise TypeError("Simulation expects a neuronbridge_gb300.SimulationConfig")
        if semantics != "auto" and semantics not in _SEMANTICS:
            raise ValueError(f"semantics must be 'auto' or one of {sorted(_SEMANTICS)}")
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
        self._dense_groups = _dense_groups(native)
        if semantics == "auto":
            semantics = _auto_semantics(native)
        self.semantics = semantics
        self._full_firing_export = [False] * len(self._dense_groups)
        self.flat = native.flat(config.timestep, _SEMANTICS[semantics], seed)
        if _instances is None:
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
        if _instances is None:
            st = self.lib.nbg_create(ctypes.byref(desc), ctypes.byref(opt), ctypes.byref(h))
        else:  # one engine over the instances (nbg_create_batch)
            made = [make_desc(p.flat(config.timestep, _SEMANTICS[semantics], seed)) for p in _instances]
            ptrs = (ctypes.POINTER(_lib.NetDesc) * len(made))(*[ctypes.pointer(m[0]) for m in made])
            first = np.zeros(len(made) + 1, np.int64)
            st = self.lib.nbg_create_batch(ptrs, len(made), ctypes.byref(opt), ctypes.byref(h),
                                           _p(first, ctypes.c_int64))
            if st == 0 and not np.array_equal(first, self.instance_first):
                raise RuntimeError("nbg_create_batch placed the instances differently from the host union")
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

    @classmethod
    def batch(cls, networks, config: SimulationConfig, **kwargs) -> "Simulation":
        """One engine over independent networks: one step loop and one launch
        per block for all of them (nbg_create_batch).  Instance k owns engine
        neurons [instance_first[k], instance_first[k + 1]) and connections
        [instance_conn_first[k], instance_conn_first[k + 1]); results per
        instance equal those of the network run alone (noisy
        IzhikevichCurrentRK4 layers excepted: their noise is keyed by the
        engine-wide neuron id)."""
        parts = [n.to_native() if isinstance(n, Network) else n for n in networks]
        if not parts or not all(isinstance(p, NetworkDescription) for p in parts):
            raise TypeError("Simulation.batch expects a non-empty list of Network or NetworkDescription")
        union, first, conn_first = NetworkDescription.concat(parts)
        sim = cls.__new__(cls)
        sim.instance_first, sim.instance_conn_first = first, conn_first
        cls.__init__(sim, union, config, _instances=parts, **kwargs)
        return sim

    @property
    def instance_count(self) -> int:
        first = getattr(self, "instance_first", None)
        return 1 if first is None else len(first) - 1

    def instance_raster(self, k: int) -> tuple[np.ndarray, np.ndarray]:
        """Spikes of instance k of a batch as (times, instance-local ids)."""
        a, b = self.instance_first[k], self.instance_first[k + 1]
        t, i = self.spike_raster()
        keep = (i >= a) & (i < b)
        return t[keep], (i[keep] - a).astype(np.int32)

    def instance_state(self, k: int, field: int) -> np.ndarray:
        return self.state_field(field)[self.instance_first[k]:self.instance_first[k + 1]]

    def instance_weights(self, k: int) -> np.ndarray:
        return self.weights()["weight"][self.instance_conn_first[k]:self.instance_conn_first[k + 1]]

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
        t0 = self.next_time
        _lib.check(self.lib.nbg_run(self._h, steps))
        self._account(self.next_time - t0)
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

    def flush(self) -> "Simulation":
        """The reference's Simulation.flush: write out the debug monitor's
        buffered rows."""
        return self.flush_debug_monitor()

    def publish_output(self) -> "Simulation":
        """The reference's publish_output pushes output spikes to its
        attached output drivers (ZeroMQ, arrays); this engine has none, and
        output_spikes() already holds every output spike, so there is nothing
        to push."""
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

    # ------------------------------------------------------ dense subnetworks
    # Layers tagged with a ``dense_subnetwork_name`` form the reference's dense
    # subnetworks (one per name, numbered in order of first appearance,
    # DenseBuildShared.cpp:655-671).  This engine runs them in its one step
    # loop with the dense runtime's semantics; these calls mirror the
    # reference's accessors (python/src/neuronbridge/__init__.py:179-181,
    # 440-469; python/bindings/neuronbridge_core.cpp:574-637).
    @property
    def dense_subnetwork_count(self) -> int:
        return len(self._dense_groups)

    def _dense_index(self, index) -> int:
        if isinstance(index, str):
            found = self.find_dense_subnetwork(index)
            if found < 0:
                raise KeyError(f"dense subnetwork was not found: {index}")
            return found
        index = int(index)
        if not 0 <= index < len(self._dense_groups):
            raise IndexError("dense subnetwork index is out of range")
        return index

    def dense_subnetwork_name(self, index: int) -> str:
        return self._dense_groups[self._dense_index(int(index))][0]

    def find_dense_subnetwork(self, name: str) -> int:
        for k, (n, _) in enumerate(self._dense_groups):
            if n == name:
                return k
        return -1

    def _dense_neurons(self, k: int) -> np.ndarray:
        start = np.concatenate([[0], np.cumsum(self.description.layer_count)])
        return np.concatenate([np.arange(start[l], start[l + 1]) for l in self._dense_groups[k][1]])

    def _dense_synapses(self, k: int) -> np.ndarray:
        inside = np.zeros(self.description.neuron_count, bool)
        inside[self._dense_neurons(k)] = True
        d = self.description
        return np.flatnonzero(inside[d.source] & inside[d.target])

    def dense_subnetwork_weights(self, index: int) -> list[float]:
        """Weights of the subnetwork's internal synapses (both ends inside it),
        in original connection order."""
        k = self._dense_index(int(index))
        return self.weights()["weight"][self._dense_synapses(k)].astype(float).tolist()

    def dense_subnetwork_snapshot(self, index) -> dict:
        """Host copy of one dense subnetwork's state (the reference's
        DenseSubnetworkDebugSnapshot as a dict).  Arrivals live in the
        engine's delay ring as bits, not in pending channels, so
        ``pending_channels`` is empty."""
        k = self._dense_index(index)
        ids = self._dense_neurons(k)
        tab = self._state_table()
        fired = (tab[_lib.FIELD_LAST_SPIKE][ids] == 0) & (self.next_time > 0)
        local_fired = np.flatnonzero(fired)
        d = self.description
        inside = np.zeros(d.neuron_count, bool)
        inside[ids] = True
        leaves = np.zeros(d.neuron_count, bool)
        leaves[d.source[inside[d.source] & ~inside[d.target]]] = True
        models = []
        for m, layer in enumerate(self._dense_groups[k][1]):
            sel = np.flatnonzero(self._layer_of[ids] == layer)
            models.append({"factory_model_id": int(d.layer_model[layer]), "model_id": m,
                           "legacy_model_name": _MODEL_NAMES.get(int(d.layer_model[layer]), ""),
                           "float_state_vectors": [tab[_lib.FIELD_V][ids[sel]].astype(float).tolist(),
                                                   tab[_lib.FIELD_U][ids[sel]].astype(float).tolist()],
                           "byte_state_vectors": []})
        return {"name": self._dense_groups[k][0], "time_step": max(self.next_time - 1, 0),
                "cuda_build_enabled": True, "gpu_backend_ready": True, "carlsim_like_gpu_active": False,
                "visible_output_firing_ids": [int(x) for x in local_fired if leaves[ids[x]]],
                "full_firing_ids": local_fired.tolist() if self._full_firing_export[k] else [],
                "membrane_v": tab[_lib.FIELD_V][ids].astype(float).tolist(),
                "gexc": tab[_lib.FIELD_G_EXC][ids].astype(float).tolist(),
                "ginh": tab[_lib.FIELD_G_INH][ids].astype(float).tolist(),
                "fired": fired.astype(int).tolist(), "pending_channels": [],
                "synaptic_weights": self.dense_subnetwork_weights(k), "synaptic_learning_pending_dwt": [],
                "model_debug_states": models, "emitted_output_spikes": [], "firing_history_ring_size": 0,
                "local_to_original_neuron_ids": ids.astype(int).tolist()}

    def reset_dense_subnetwork(self, index) -> "Simulation":
        """Initial state for the subnetwork's neurons and no pending arrivals
        for them; weights, traces and time are kept."""
        k = self._dense_index(index)
        start = np.concatenate([[0], np.cumsum(self.description.layer_count)])
        for layer in self._dense_groups[k][1]:
            _lib.check(self.lib.nbg_reset_neurons(self._h, int(start[layer]),
                                                   int(self.description.layer_count[layer])))
        return self

    def set_dense_subnetwork_full_firing_export_enabled(self, index, enabled: bool = True) -> "Simulation":
        self._full_firing_export[self._dense_index(index)] = bool(enabled)
        return self

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
        """Device timings (CUDA events on the engine stream): the last run
        call's, and the totals since construction or reset_bench_profiling.
        The reference's snapshot splits its host event loop into phases
        (python/bindings/neuronbridge_core.cpp:40-90); this engine has no host
        loop, so the figures are the device time of the step loop."""
        tot, upd, prop = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        n = ctypes.c_int64()
        _lib.check(self.lib.nbg_profile(self._h, ctypes.byref(tot), ctypes.byref(upd), ctypes.byref(prop),
                                        ctypes.byref(n)))
        acc = getattr(self, "_prof_total", None) or {"total_device_ms": 0.0, "total_kernel_launches": 0,
                                                     "run_calls": 0, "simulated_steps": 0}
        ro, rd, ra = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        rn = ctypes.c_int64()
        _lib.check(self.lib.nbg_raster_profile(self._h, ctypes.byref(ro), ctypes.byref(rd), ctypes.byref(ra),
                                               ctypes.byref(rn)))
        return {"device_ms": tot.value, "update_kernel_ms": upd.value, "propagate_kernel_ms": prop.value,
                "kernel_launches": n.value, "raster_order_ms": ro.value, "raster_order_launches": rn.value,
                "raster_download_ms": rd.value, "raster_append_ms": ra.value, **acc}

    def reset_bench_profiling(self) -> "Simulation":
        """Zero the totals of bench_profiling_snapshot."""
        self._prof_total = {"total_device_ms": 0.0, "total_kernel_launches": 0, "run_calls": 0,
                            "simulated_steps": 0}
        return self

    def _account(self, steps: int) -> None:
        if getattr(self, "_prof_total", None) is None:
            self.reset_bench_profiling()
        tot, n = ctypes.c_double(), ctypes.c_int64()
        _lib.check(self.lib.nbg_profile(self._h, ctypes.byref(tot), None, None, ctypes.byref(n)))
        acc = self._prof_total
        acc["total_device_ms"] += tot.value
        acc["total_kernel_launches"] += n.value
        acc["run_calls"] += 1
        acc["simulated_steps"] += steps
