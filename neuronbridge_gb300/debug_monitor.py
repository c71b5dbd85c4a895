"""DebugMonitor: CSV records of neuron state, spikes and weights.

Mirrors the reference's main-network monitor (python/src/neuronbridge/
config.py:15-67 ``DebugMonitorConfig``, results.py:12-72
``DebugMonitorResult``; src/native/gpu/src/debug_monitor/
DebugMonitorWriter.cpp, MainNetworkDebugSource.cpp, SimulationDebugMonitor.cpp):

* enabling it creates the output directory, ``meta.json`` and the eight CSV
  files; headers are written with the first frame;
* a frame is captured at the end of every ``run`` call (the reference calls
  ``CaptureDebugMonitorStep(currenttime)`` once at the end of
  ``RunSimulationStep``), at time step = the last step the call updated, and
  only when that step is a multiple of ``sample_interval_steps``;
* state rows: every printable value of each selected neuron -- the model's
  state variables, then ``LastUpdate`` and two -1 placeholders
  (Neuron_State_Vector::GetPrintableValuesAt); field 0 is named ``v``,
  field k ``state_k``; values printed as C++ ``operator<<`` does (%g);
* spike rows: every spike of a selected neuron since the previous frame
  (Simulation::WriteSpike feeds the monitor for each spike, whatever its
  time), in raster order;
* weight rows: all main-network weights in original connection order;
* files are flushed every ``flush_interval_steps`` frames and on
  ``flush_debug_monitor``.

Selected neurons: all (``all_neurons``), else ``neuron_ids``, else the
neurons of layers declared ``monitored``.  The engine records the raster of
the layers holding selected neurons in addition to the output layers; the
spikes are read back once per run call, so nothing runs per step on the host.
Dense subnetworks, InputConv and OuterDynamic sources are not part of this
engine: their files are created with headers only.
"""
from __future__ import annotations

import csv
import ctypes
import json
from dataclasses import dataclass, field
from pathlib import Path
from typing import Iterator

import numpy as np

from . import _lib

_HEADERS = {
    "neuron_state.csv": "time_step,component_kind,component_index,component_name,global_neuron_id,local_neuron_id,"
                        "field_name,value",
    "spikes.csv": "time_step,component_kind,component_index,component_name,global_neuron_id,local_neuron_id",
    "pending_channels.csv": "time_step,subnetwork_index,subnetwork_name,channel,local_neuron_id,global_neuron_id,"
                            "value",
    "inputconv_outputs.csv": "time_step,inputconv_index,inputconv_name,output_index,value",
    "inputconv_inputs.csv": "time_step,inputconv_index,inputconv_name,input_index,value",
    "inputconv_state.csv": "time_step,inputconv_index,inputconv_name,field_name,state_index,value",
    "outer_dynamic_state.csv": "time_step,component_index,component_name,field_name,index,value",
    "weights.csv": "time_step,component_kind,component_index,component_name,synapse_id,value",
}
_MAIN = "main_network,0,main_network"

# engine state field of each printable state variable, per model (None: the
# variable exists in the reference's state vector but this engine keeps it 0)
_FIELDS = {
    _lib.MODEL_LIF_VJ: [0, 4],                   # V, I_ext
    _lib.MODEL_IZH_COND: [0, 1, 2, 3, None, 4],  # v, u, g_ampa, g_gaba, g_nmda, I_ext
    _lib.MODEL_IZH_RK4: [0, 1, 4],               # v, u, I_bias (this engine's model)
    _lib.MODEL_POISSON: [None, 4],               # rate increment (reset by every update), I_ext
}


def _g(x: float) -> str:
    """C++ default ostream formatting of a float (six significant digits)."""
    s = "%g" % x
    return "-0" if s == "-0" else s


@dataclass
class DebugMonitorConfig:
    enabled: bool = True
    output_dir: str | Path = "debug_monitor"
    sample_interval_steps: int = 1
    flush_interval_steps: int = 100
    record_spikes: bool = True
    record_state: bool = True
    record_weights: bool = False
    record_pending_channels: bool = True
    record_outer_dynamic_state: bool = True
    all_neurons: bool = False
    neuron_ids: list = field(default_factory=list)
    dense_local_neuron_ids: dict = field(default_factory=dict)
    record_inputconv_outputs: bool = True
    record_inputconv_inputs: bool = False
    record_inputconv_internal_state: bool = False
    monitor_all_inputconv: bool = False
    monitored_inputconv_indices: list = field(default_factory=list)
    monitored_inputconv_names: list = field(default_factory=list)

    def to_dict(self) -> dict:
        return {k: (str(v) if k == "output_dir" else v) for k, v in self.__dict__.items()}


class DebugMonitorResult:
    """Lazy access to the CSV/JSON files of a monitor directory."""

    KNOWN_TABLES = {
        "neuron_state": "neuron_state.csv", "pending_channels": "pending_channels.csv", "spikes": "spikes.csv",
        "weights": "weights.csv", "outer_dynamic_state": "outer_dynamic_state.csv",
        "inputconv_outputs": "inputconv_outputs.csv", "inputconv_inputs": "inputconv_inputs.csv",
        "inputconv_state": "inputconv_state.csv",
    }

    def __init__(self, path):
        self.path = Path(path)
        if not self.path.exists():
            raise FileNotFoundError(self.path)
        if not self.path.is_dir():
            raise NotADirectoryError(self.path)

    @property
    def meta_path(self) -> Path:
        return self.path / "meta.json"

    def meta(self) -> dict:
        return json.loads(self.meta_path.read_text(encoding="utf-8")) if self.meta_path.exists() else {}

    def table_path(self, name: str) -> Path:
        path = self.path / self.KNOWN_TABLES.get(name, name)
        if not path.exists():
            raise FileNotFoundError(path)
        return path

    def iter_rows(self, name: str, *, limit: int | None = None) -> Iterator[dict]:
        with self.table_path(name).open("r", encoding="utf-8", newline="") as handle:
            for count, row in enumerate(csv.DictReader(handle)):
                if limit is not None and count >= limit:
                    return
                yield row

    def to_pandas(self, name: str, **kwargs):
        import pandas as pd

        return pd.read_csv(self.table_path(name), **kwargs)

    def file_sizes(self) -> dict:
        return {t: (self.path / f).stat().st_size for t, f in self.KNOWN_TABLES.items() if (self.path / f).exists()}


def open_debug_monitor(path) -> DebugMonitorResult:
    return DebugMonitorResult(path)


class DebugMonitor:
    """The monitor attached to one Simulation (see the module docstring)."""

    def __init__(self, sim, config: DebugMonitorConfig):
        if not str(config.output_dir):
            raise ValueError("debug monitor output_dir must not be empty")
        self.sim = sim
        self.config = config
        self.interval = max(1, int(config.sample_interval_steps))
        self.flush_every = int(config.flush_interval_steps) if config.flush_interval_steps > 0 else 100
        self.root = Path(config.output_dir)
        self.root.mkdir(parents=True, exist_ok=True)
        self.files = {name: (self.root / name).open("w", encoding="utf-8", newline="") for name in _HEADERS}
        self.headers = False
        (self.root / "meta.json").write_text(
            "{\n"
            f'  "sample_interval_steps": {config.sample_interval_steps},\n'
            f'  "flush_interval_steps": {config.flush_interval_steps},\n'
            f'  "record_state": {str(config.record_state).lower()},\n'
            f'  "record_spikes": {str(config.record_spikes).lower()},\n'
            f'  "record_weights": {str(config.record_weights).lower()},\n'
            f'  "record_pending_channels": {str(config.record_pending_channels).lower()},\n'
            f'  "record_inputconv_outputs": {str(config.record_inputconv_outputs).lower()},\n'
            f'  "record_outer_dynamic_state": {str(config.record_outer_dynamic_state).lower()}\n'
            "}\n", encoding="utf-8")
        d = sim.description
        n = d.neuron_count
        layer_of = np.repeat(np.arange(len(d.layer_count)), d.layer_count)
        if config.all_neurons:
            sel = np.ones(n, bool)
        elif config.neuron_ids:
            sel = np.zeros(n, bool)
            ids = np.asarray(config.neuron_ids, np.int64)
            sel[ids[(ids >= 0) & (ids < n)]] = True
        else:
            sel = np.repeat(np.asarray(sim._layer_monitored, bool), d.layer_count)
        self.selected = sel
        self.ids = np.flatnonzero(sel)
        self.layer_of = layer_of
        self.models = d.layer_model[layer_of[self.ids]] if len(self.ids) else np.zeros(0, np.int32)
        # the raster must hold every selected neuron's spikes
        if config.record_spikes:
            for layer in np.unique(layer_of[self.ids]):
                if not d.layer_output[layer]:
                    _lib.check(sim.lib.nbg_set_layer_record(sim._h, int(layer), 1))
                    sim._extra_recorded = True
        self.read = sim._num_raster()  # raster entries already seen
        self.pending: list[str] = []
        self.frames_since_flush = 0

    def _write_headers(self) -> None:
        if not self.headers:
            for name, header in _HEADERS.items():
                self.files[name].write(header + "\n")
            self.headers = True

    def collect_spikes(self) -> None:
        """Move the spikes the last run call recorded into the pending list."""
        total = self.sim._num_raster()
        if total > self.read and self.config.record_spikes:
            t, i = self.sim._raster_range(self.read, total - self.read)
            keep = self.selected[i]
            self.pending.extend(f"{a},{_MAIN},{b},{b}\n" for a, b in zip(t[keep].tolist(), i[keep].tolist()))
        self.read = total

    def capture(self, time_step: int) -> None:
        self.collect_spikes()
        if self.interval > 1 and time_step % self.interval != 0:
            return
        rows = []
        if self.config.record_state and len(self.ids):
            cache = {}
            for m in np.unique(self.models):
                sel = self.ids[self.models == m]
                fields = _FIELDS.get(int(m))
                if fields is None:  # event-driven input layers: no state vector
                    continue
                vals = []
                for f in fields:
                    if f is None:
                        vals.append(np.zeros(len(sel), np.float32))
                        continue
                    if f not in cache:
                        cache[f] = self.sim.state_field(f)
                    vals.append(cache[f][sel])
                cols = len(fields)
                for k, j in enumerate(sel.tolist()):
                    prefix = f"{time_step},{_MAIN},{j},{j},"
                    for c in range(cols):
                        rows.append(f"{prefix}{'v' if c == 0 else f'state_{c}'},{_g(float(vals[c][k]))}\n")
                    rows.append(f"{prefix}state_{cols},{_g(float(time_step))}\n")  # LastUpdate
                    rows.append(f"{prefix}state_{cols + 1},-1\n")
                    rows.append(f"{prefix}state_{cols + 2},-1\n")
        weights = []
        if self.config.record_weights:
            w = self.sim.weights()["weight"]
            weights = [f"{time_step},{_MAIN},{s},{_g(float(x))}\n" for s, x in enumerate(w.tolist())]
        if rows or self.pending or weights:
            self._write_headers()
            self.files["neuron_state.csv"].writelines(rows)
            self.files["spikes.csv"].writelines(self.pending)
            self.files["weights.csv"].writelines(weights)
            self.pending = []
        self.frames_since_flush += 1
        if self.frames_since_flush >= self.flush_every:
            self.frames_since_flush = 0
            self.flush_files()

    def flush_files(self) -> None:
        for f in self.files.values():
            f.flush()

    def flush(self) -> None:
        self.collect_spikes()
        if self.pending:
            self._write_headers()
            self.files["spikes.csv"].writelines(self.pending)
            self.pending = []
        self.flush_files()

    def close(self) -> None:
        self.flush()
        for f in self.files.values():
            f.close()
