"""Network description objects with the reference's Python API shape.

Mirrors ``python/src/neuronbridge/model.py`` of the reference (``NeuronLayer``
:145-238, ``Connection`` :241-290, ``LearningRule`` :293-302,
``SimulationConfig`` :755-790, ``Network`` :793-912): same class names, field
names, defaults and validation errors, so network-building code written for
the reference runs unchanged.  ``Network.to_native()`` produces a
:class:`NetworkDescription` of flat arrays instead of a pybind11 object; it is
what crosses the C ABI (``include/nbg.h``, ``nbg_net_desc``).

GB300 additions: ``Connection`` also accepts numpy arrays (10^7-synapse
networks are built without Python lists), and the current-based RK4
Izhikevich model ``IzhikevichCurrentRK4`` is registered beside the
reference's models.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Any

import numpy as np

from . import _lib

ParameterScalar = bool | int | float | str


@dataclass(frozen=True, slots=True)
class NativeParameter:
    """Typed parameter value (the reference's ``NativeParameter``, model.py:18-40)."""

    kind: str
    value: Any

    def __post_init__(self) -> None:
        valid = {"int32", "float32", "float64", "int32_list", "float32_list", "float64_list", "float32_array3",
                 "float32_array4", "float32_array5"}
        if self.kind not in valid:
            raise ValueError(f"unsupported native parameter kind: {self.kind}")


def int32(value: int) -> NativeParameter:
    return NativeParameter("int32", int(value))


def float32(value: float) -> NativeParameter:
    return NativeParameter("float32", float(value))


def float64(value: float) -> NativeParameter:
    return NativeParameter("float64", float(value))


def float32_list(values) -> NativeParameter:
    return NativeParameter("float32_list", [float(v) for v in values])


def _plain(value):
    return value.value if isinstance(value, NativeParameter) else value


def _validate_parameters(parameters: dict) -> dict:
    out = {}
    for key, value in parameters.items():
        if not isinstance(key, str):
            raise TypeError("parameter names must be strings")
        if not isinstance(value, (NativeParameter, bool, int, float, str, list)):
            raise TypeError(f"unsupported parameter type for {key!r}: {type(value).__name__}")
        out[key] = value
    return out


# ---------------------------------------------------------------- model catalog
# canonical name -> (model id, aliases); names and aliases as the reference's
# src/native/shared/src/neuron_model/NeuronModelCatalog.cpp:60-200
CATALOG = {
    "TimeDrivenLIF_Voltage_jump": (_lib.MODEL_LIF_VJ, ("TimeDrivenLIF_Voltage_jump_GPU",)),
    "TimeDrivenIzhikevic_Exponential_Decay": (
        _lib.MODEL_IZH_COND,
        ("TimeDrivenIzhikevic_I_Exponential_Decay", "TimeDrivenIzhikevic_I_Exponential_Decay_GPU",
         "TimeDrivenIzhikevic_Exponential_Decay_GPU")),
    "PoissonRate": (_lib.MODEL_POISSON, ("PoissonRate_GPU",)),
    "IzhikevichCurrentRK4": (_lib.MODEL_IZH_RK4, ()),
    "InputSpikeNeuronModel": (_lib.MODEL_INPUT_SPIKE, ()),
    "InputCurrentNeuronModel": (_lib.MODEL_INPUT_CURRENT, ()),
}
_ALIAS = {alias: canon for canon, (_, aliases) in CATALOG.items() for alias in (canon, *aliases)}

# parameter name -> (slot kind, slot index, default); defaults are the
# reference model headers' member initialisers
_PARAMS = {
    _lib.MODEL_LIF_VJ: {  # TimeDrivenLIF_Voltage_jump.h:22-32
        "V_rest": ("f", 0, 0.0), "tau": ("f", 1, 10.0), "V_th": ("f", 2, 20.0), "R": ("f", 3, 1.0),
        "V_reset": ("f", 4, -5.0), "random_mu": ("f", 5, 0.0), "I_ext": ("f", 6, 0.0), "t_ref": ("i", 0, 50),
    },
    _lib.MODEL_IZH_COND: {  # TimeDrivenIzhikevic_Exponential_Decay.h:28-52
        "a": ("f", 0, 0.02), "b": ("f", 1, 0.2), "c": ("f", 2, -65.0), "d": ("f", 3, 8.0),
        "V_rest": ("f", 4, -65.0), "V_th": ("f", 5, 30.0), "R": ("f", 6, 1.0), "E_ampa": ("f", 7, 0.0),
        "ampa_tau": ("f", 8, 5.0), "E_gaba": ("f", 9, -80.0), "gaba_tau": ("f", 10, 10.0),
        "I_ext": ("f", 11, 0.0), "V_reset": (None, 0, -65.0), "nmda_tau": (None, 0, 100.0),
    },
    _lib.MODEL_IZH_RK4: {
        "a": ("f", 0, 0.02), "b": ("f", 1, 0.2), "c": ("f", 2, -65.0), "d": ("f", 3, 8.0),
        "v0": ("f", 4, -65.0), "V_th": ("f", 5, 30.0), "noise_sigma": ("f", 6, 0.0), "I_bias": ("f", 7, 0.0),
    },
    _lib.MODEL_POISSON: {  # PoissonRate.h:12-13, PoissonRate.cpp:133-150
        "rate_bias_hz": ("f", 0, 0.0), "poisson_rate_bias_hz": ("f", 0, 0.0),
        "rate_gain_hz_per_current": ("f", 1, 1.0), "poisson_rate_gain_hz_per_current": ("f", 1, 1.0),
        "I_ext": ("f", 2, 0.0),
    },
    _lib.MODEL_INPUT_SPIKE: {},
    _lib.MODEL_INPUT_CURRENT: {},
}


def resolve_model(name: str) -> int:
    canon = _ALIAS.get(name)
    if canon is None:
        raise ValueError(f"neuron model {name!r} is not supported by the GB300 engine "
                         f"(supported: {', '.join(sorted(_ALIAS))})")
    return CATALOG[canon][0]


@dataclass(slots=True)
class NeuronLayer:
    model: str
    count: int
    update_timestep: int = 1
    monitored: bool = False
    output: bool = False
    communication_input: bool = False
    parameters: dict = field(default_factory=dict)

    def __post_init__(self) -> None:
        if self.count <= 0:
            raise ValueError("NeuronLayer.count must be positive")
        if self.update_timestep <= 0:
            raise ValueError("NeuronLayer.update_timestep must be positive")
        self.parameters = _validate_parameters(dict(self.parameters))

    @classmethod
    def poisson_rate(cls, count: int, *, dense_name: str | None = None, rate_bias_hz: float | None = None,
                     rate_gain_hz_per_current: float | None = None, update_timestep: int = 1,
                     monitored: bool = False, output: bool = False, communication_input: bool = False,
                     **parameters) -> "NeuronLayer":
        params = dict(parameters)
        if dense_name is not None:
            params["dense_subnetwork_name"] = dense_name
        if rate_bias_hz is not None:
            params["poisson_rate_bias_hz"] = float32(rate_bias_hz)
        if rate_gain_hz_per_current is not None:
            params["poisson_rate_gain_hz_per_current"] = float32(rate_gain_hz_per_current)
        return cls("PoissonRate", count, update_timestep=update_timestep, monitored=monitored, output=output,
                   communication_input=communication_input, parameters=params)

    @classmethod
    def input_spike(cls, count: int, *, update_timestep: int = 1, monitored: bool = False, output: bool = False,
                    communication_input: bool = False, **parameters) -> "NeuronLayer":
        """Event-driven layer whose neurons spike only through
        Simulation.add_external_spikes (reference model.py:162-172)."""
        return cls("InputSpikeNeuronModel", count, update_timestep=update_timestep, monitored=monitored,
                   output=output, communication_input=communication_input, parameters=dict(parameters))

    @classmethod
    def input_current(cls, count: int, *, update_timestep: int = 1, monitored: bool = False, output: bool = False,
                      communication_input: bool = False, **parameters) -> "NeuronLayer":
        """Event-driven layer whose neurons send Simulation.add_external_currents
        over their current synapses (synapse_type=3; reference model.py:174-185)."""
        return cls("InputCurrentNeuronModel", count, update_timestep=update_timestep, monitored=monitored,
                   output=output, communication_input=communication_input, parameters=dict(parameters))

    def native_params(self) -> tuple[int, np.ndarray, np.ndarray]:
        """(model id, f[16], ip[4]) for the C ABI layer descriptor."""
        if self.update_timestep != 1:
            raise ValueError("the GB300 engine integrates every layer every step (update_timestep must be 1)")
        mid = resolve_model(self.model)
        table = _PARAMS[mid]
        f = np.zeros(_lib.NFP, np.float32)
        ip = np.zeros(_lib.NIP, np.int32)
        for _, (kind, idx, default) in table.items():
            if kind == "f":
                f[idx] = default
            elif kind == "i":
                ip[idx] = default
        for key, value in self.parameters.items():
            value = _plain(value)
            if key in ("dense_subnetwork_name", "int_method"):
                continue
            if key == "random_sigma":
                if any(float(x) != 0.0 for x in np.atleast_1d(value)):
                    raise ValueError("random_sigma must be 0: the reference draws it from std::random_device, "
                                     "which is not reproducible")
                continue
            if key not in table:
                raise ValueError(f"unknown parameter {key!r} for model {self.model!r}")
            kind, idx, _ = table[key]
            if kind is None:
                continue
            if key == "random_mu":
                value = np.atleast_1d(value)[0]
            if kind == "f":
                f[idx] = np.float32(value)
            else:
                ip[idx] = int(value)
        return mid, f, ip

    def to_dict(self) -> dict:
        return {"model": self.model, "count": self.count, "update_timestep": self.update_timestep,
                "monitored": self.monitored, "output": self.output, "communication_input": self.communication_input,
                "parameters": {k: _plain(v) for k, v in self.parameters.items()}}


def _as_array(value, dtype, name):
    if isinstance(value, np.ndarray):
        return value.astype(dtype, copy=False).ravel()
    if isinstance(value, (list, tuple)):
        return np.asarray(value, dtype=dtype)
    return np.asarray([value], dtype=dtype)


@dataclass(slots=True)
class Connection:
    source: Any
    target: Any
    synapse_type: Any = 0
    weight: Any = 1.0
    max_weight: Any = None
    delay: Any = 1
    synapse_rule: Any = -1
    trigger_rule: Any = -1

    def normalized(self) -> dict:
        source = _as_array(self.source, np.int32, "source")
        target = _as_array(self.target, np.int32, "target")
        count = max(len(source), len(target))
        if len(source) == 1 and count > 1:
            source = np.repeat(source, count)
        if len(target) == 1 and count > 1:
            target = np.repeat(target, count)
        if len(source) != len(target):
            raise ValueError("Connection.source and target lengths must match or be scalar")

        def expand(value, dtype, name):
            arr = _as_array(value, dtype, name)
            if len(arr) == 1 and count > 1:
                arr = np.repeat(arr, count)
            if len(arr) != count:
                raise ValueError(f"Connection.{name} length must be 1 or {count}")
            return arr

        weight = expand(self.weight, np.float32, "weight")
        return {
            "source": source, "target": target,
            "synapse_type": expand(self.synapse_type, np.int32, "synapse_type"),
            "weight": weight,
            "max_weight": expand(self.weight if self.max_weight is None else self.max_weight, np.float32,
                                 "max_weight"),
            "delay": expand(self.delay, np.int32, "delay"),
            "synapse_rule": expand(self.synapse_rule, np.int32, "synapse_rule"),
            "trigger_rule": expand(self.trigger_rule, np.int32, "trigger_rule"),
        }

    def to_dict(self) -> dict:
        return {k: v.tolist() for k, v in self.normalized().items()}


# STDP defaults: the reference's STDP.h:14-20
_STDP_DEFAULTS = {"Max_LTP": 0.92, "LTP_tau": 16.8, "Max_LTD": 0.53, "LTD_tau": 33.1}


@dataclass(slots=True)
class LearningRule:
    name: str
    parameters: dict = field(default_factory=dict)

    def __post_init__(self) -> None:
        self.parameters = _validate_parameters(dict(self.parameters))

    def native_params(self) -> np.ndarray:
        if self.name != "STDP":
            raise ValueError(f"learning rule {self.name!r} is not supported by the GB300 engine (supported: STDP)")
        p = dict(_STDP_DEFAULTS)
        for k, v in self.parameters.items():
            if k not in p:
                raise ValueError(f"unknown STDP parameter {k!r}")
            p[k] = float(_plain(v))
        return np.array([p["Max_LTP"], p["LTP_tau"], p["Max_LTD"], p["LTD_tau"]], np.float32)

    def to_dict(self) -> dict:
        return {"name": self.name, "parameters": {k: _plain(v) for k, v in self.parameters.items()}}


@dataclass(slots=True)
class SimulationConfig:
    steps: int
    timestep: float
    queues: int = 1
    event_queue: str = "heap"
    timing_wheel_size: int = 0

    def __post_init__(self) -> None:
        if self.steps <= 0:
            raise ValueError("SimulationConfig.steps must be positive")
        if self.timestep <= 0:
            raise ValueError("SimulationConfig.timestep must be positive")
        if self.queues <= 0:
            raise ValueError("SimulationConfig.queues must be positive")
        if self.event_queue not in {"heap", "timing_wheel"}:
            raise ValueError("SimulationConfig.event_queue must be 'heap' or 'timing_wheel'")

    def to_dict(self) -> dict:
        return {"steps": self.steps, "timestep": self.timestep, "queues": self.queues,
                "event_queue": self.event_queue, "timing_wheel_size": self.timing_wheel_size}


# models the reference's dense GPU runtime implements among this engine's
# (NeuronModelCatalog.cpp: the DenseGpu bindings)
DENSE_MODELS = (_lib.MODEL_LIF_VJ, _lib.MODEL_IZH_COND, _lib.MODEL_POISSON)


def dense_name_of(layer: "NeuronLayer") -> str | None:
    """The layer's dense subnetwork (its ``dense_subnetwork_name`` parameter),
    validated as the reference's dense build does
    (src/native/gpu/src/simulation_dense/DenseBuildShared.cpp:169-197, 649-653):
    input models stay in the main network, a dense layer is not an output
    layer, and its model must have a dense GPU implementation."""
    name = layer.parameters.get("dense_subnetwork_name")
    if name is None:
        return None
    name = str(_plain(name))
    if not name:
        return None
    mid = resolve_model(layer.model)
    if mid in (_lib.MODEL_INPUT_SPIKE, _lib.MODEL_INPUT_CURRENT):
        raise RuntimeError(f"Input neuron model '{layer.model}' cannot be placed inside dense subnetwork "
                           f"'{name}'; declare it in the main network and connect it to dense target neurons "
                           "instead.")
    if mid not in DENSE_MODELS:
        raise RuntimeError(f"Neuron model '{layer.model}' is not supported by dense GPU subnetwork '{name}'.")
    if layer.output:
        raise RuntimeError("dense subnetwork layer cannot be marked isOutput=true; declare dense outputs by "
                           "adding dense->main or dense->dense connections")
    return name


class NetworkDescription:
    """Flat, C-ABI-ready description (the counterpart of ``_core.NetworkDescription``)."""

    def __init__(self, layers: list[NeuronLayer], connections: list[Connection], rules: list[LearningRule]):
        n = len(layers)
        self.layer_model = np.zeros(n, np.int32)
        self.layer_count = np.zeros(n, np.int32)
        self.layer_fparams = np.zeros((n, _lib.NFP), np.float32)
        self.layer_iparams = np.zeros((n, _lib.NIP), np.int32)
        self.layer_output = np.zeros(n, bool)
        self.layer_monitored = np.zeros(n, bool)
        self.layer_dense: list[str | None] = []  # dense_subnetwork_name of each layer (None: main network)
        for i, layer in enumerate(layers):
            mid, f, ip = layer.native_params()
            self.layer_model[i] = mid
            self.layer_count[i] = layer.count
            self.layer_fparams[i] = f
            self.layer_iparams[i] = ip
            self.layer_output[i] = layer.output
            self.layer_monitored[i] = layer.monitored
            self.layer_dense.append(dense_name_of(layer))
        parts = [c.normalized() for c in connections]
        cat = lambda key, dt: (np.concatenate([p[key] for p in parts]).astype(dt, copy=False)
                               if parts else np.zeros(0, dt))
        self.source = cat("source", np.int32)
        self.target = cat("target", np.int32)
        self.type = cat("synapse_type", np.int32)
        self.weight = cat("weight", np.float32)
        self.max_weight = cat("max_weight", np.float32)
        self.delay = cat("delay", np.int32)
        self.rule = cat("synapse_rule", np.int32)
        trig = cat("trigger_rule", np.int32)
        if len(trig) and np.any(trig != -1):
            raise ValueError("trigger rules are not supported by the GB300 engine")
        self.rule_params = (np.stack([r.native_params() for r in rules]) if rules
                            else np.zeros((0, 4), np.float32))

    @classmethod
    def from_arrays(cls, layers: list[NeuronLayer], source, target, synapse_type, weight, max_weight=None,
                    delay=1, synapse_rule=-1, rules: list[LearningRule] | None = None) -> "NetworkDescription":
        """Build directly from flat connection arrays (original connection
        order = array order), without Connection objects."""
        d = cls(layers, [], rules or [])
        n = len(source)

        def arr(x, dt):
            a = np.asarray(x, dtype=dt)
            return np.full(n, a, dtype=dt) if a.ndim == 0 else np.ascontiguousarray(a.ravel())

        d.source = arr(source, np.int32)
        d.target = arr(target, np.int32)
        d.type = arr(synapse_type, np.int32)
        d.weight = arr(weight, np.float32)
        d.max_weight = d.weight.copy() if max_weight is None else arr(max_weight, np.float32)
        d.delay = arr(delay, np.int32)
        d.rule = arr(synapse_rule, np.int32)
        if not (len(d.target) == len(d.type) == len(d.weight) == len(d.delay) == len(d.rule) == n):
            raise ValueError("connection arrays must have one entry per connection")
        return d

    @classmethod
    def concat(cls, parts: list["NetworkDescription"]) -> tuple["NetworkDescription", np.ndarray, np.ndarray]:
        """Independent networks as one description (the host form of
        nbg_create_batch): layers, connections and learning rules
        concatenated, neuron ids of part k offset by the neurons of parts
        0..k-1 and its rule ids by their rules.  Returns (union, first
        neuron of each part + total, first connection of each part + total)."""
        if not parts:
            raise ValueError("need at least one network")
        d = cls([], [], [])
        neurons = np.array([0] + [p.neuron_count for p in parts], np.int64).cumsum()
        conns = np.array([0] + [len(p.source) for p in parts], np.int64).cumsum()
        rules = np.array([0] + [len(p.rule_params) for p in parts], np.int64).cumsum()
        for key in ("layer_model", "layer_count", "layer_fparams", "layer_iparams", "layer_output", "layer_monitored"):
            setattr(d, key, np.concatenate([getattr(p, key) for p in parts]))
        d.layer_dense = [name for p in parts for name in getattr(p, "layer_dense", [None] * len(p.layer_count))]
        d.source = np.concatenate([p.source + neurons[k] for k, p in enumerate(parts)]).astype(np.int32)
        d.target = np.concatenate([p.target + neurons[k] for k, p in enumerate(parts)]).astype(np.int32)
        for key in ("type", "weight", "max_weight", "delay"):
            setattr(d, key, np.concatenate([getattr(p, key) for p in parts]))
        d.rule = np.concatenate([np.where(p.rule >= 0, p.rule + rules[k], p.rule)
                                 for k, p in enumerate(parts)]).astype(np.int32)
        d.rule_params = (np.concatenate([p.rule_params for p in parts]).astype(np.float32) if rules[-1]
                         else np.zeros((0, 4), np.float32))
        return d, neurons, conns

    @property
    def neuron_count(self) -> int:
        return int(self.layer_count.sum())

    def flat(self, dt: float, semantics: int = _lib.SEM_LEGACY_CPU, seed: int = 0) -> dict:
        return {"layer_model": self.layer_model, "layer_count": self.layer_count, "layer_output": self.layer_output,
                "layer_fparams": self.layer_fparams, "layer_iparams": self.layer_iparams,
                "source": self.source, "target": self.target, "type": self.type, "weight": self.weight,
                "max_weight": self.max_weight, "delay": self.delay, "rule": self.rule,
                "rule_params": self.rule_params, "dt": float(dt), "semantics": int(semantics), "seed": int(seed)}


@dataclass(slots=True)
class Network:
    layers: list = field(default_factory=list)
    connections: list = field(default_factory=list)
    learning_rules: list = field(default_factory=list)

    def add_layer(self, layer: NeuronLayer) -> "Network":
        if not isinstance(layer, NeuronLayer):
            raise TypeError("Network.add_layer expects a NeuronLayer")
        self.layers.append(layer)
        return self

    def connect(self, connection: Connection) -> "Network":
        if not isinstance(connection, Connection):
            raise TypeError("Network.connect expects a Connection")
        self.connections.append(connection)
        return self

    def add_learning_rule(self, rule: LearningRule) -> "Network":
        if not isinstance(rule, LearningRule):
            raise TypeError("Network.add_learning_rule expects a LearningRule")
        self.learning_rules.append(rule)
        return self

    @property
    def neuron_count(self) -> int:
        return sum(layer.count for layer in self.layers)

    def to_native(self) -> NetworkDescription:
        return NetworkDescription(self.layers, self.connections, self.learning_rules)

    def to_dict(self) -> dict:
        return {"layers": [l.to_dict() for l in self.layers],
                "connections": [c.to_dict() for c in self.connections],
                "learning_rules": [r.to_dict() for r in self.learning_rules]}
