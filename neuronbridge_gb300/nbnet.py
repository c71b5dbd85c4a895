"""``.nbnet`` network files: authoring, validation and bounded-memory loading.

The format is the reference's (python/src/neuronbridge/nbnet.py:35-42,
src/native/shared/src/streaming_build/NbnetReader.cpp), so files written by
either side load in the other:

* header, little-endian ``<8sHHIIQQ32s``: magic ``NBNET01\\0``, version
  major 1 / minor 0, flags (bit 0: SHA-256 present), connection record size
  (32), metadata size, connection count, SHA-256 of metadata + records;
* metadata: UTF-8 JSON (sorted keys, no spaces) with ``layers``,
  ``learning_rules``, ``outer_dynamics``, ``outer_dynamic_connections`` and
  ``input_convs``; parameter values carry their kind
  (``{"__neuronbridge_parameter__": kind, "value": v}``);
* connection records, ``<IIiffIii``: source, target, synapse type, weight,
  max weight, delay, synapse rule, trigger rule, in original connection order.

Writing is vectorised (one numpy record array per batch, spooled to disk).
Loading maps the record block (``numpy.memmap``) and fills the engine's flat
int32/float32 connection columns in batches bounded by the memory budget, so
no per-connection Python object is ever made; the engine then builds its CSC
directly from those columns.
"""
from __future__ import annotations

import hashlib
import json
import math
import os
import struct
import tempfile
import time
from dataclasses import dataclass
from pathlib import Path
from typing import Any, Iterable, Mapping

import numpy as np

from .model import Connection, LearningRule, NativeParameter, Network, NetworkDescription, NeuronLayer

MAGIC = b"NBNET01\0"
VERSION_MAJOR, VERSION_MINOR = 1, 0
HEADER = struct.Struct("<8sHHIIQQ32s")
RECORD = np.dtype([("source", "<u4"), ("target", "<u4"), ("synapse_type", "<i4"), ("weight", "<f4"),
                   ("max_weight", "<f4"), ("delay", "<u4"), ("synapse_rule", "<i4"), ("trigger_rule", "<i4")])
FLAG_SHA256 = 1
PARAMETER_MARKER = "__neuronbridge_parameter__"
MAX_METADATA_BYTES = 64 * 1024 * 1024
_NATIVE_KINDS = {"int32", "float32", "float64", "int32_list", "float32_list", "float64_list", "float32_array3",
                 "float32_array4", "float32_array5"}
assert RECORD.itemsize == 32


@dataclass(frozen=True, slots=True)
class StreamingBuildOptions:
    """Bounded-memory loading of a ``.nbnet`` description."""

    memory_budget_mb: int = 128
    mmap: bool = True
    verify_checksum: bool = True

    def __post_init__(self) -> None:
        if self.memory_budget_mb <= 0:
            raise ValueError("memory_budget_mb must be positive")


@dataclass(frozen=True, slots=True)
class NbnetWriteOptions:
    overwrite: bool = False
    fsync: bool = True


@dataclass(frozen=True, slots=True)
class NbnetLayerHandle:
    index: int
    first_neuron_id: int
    count: int


@dataclass(frozen=True, slots=True)
class NbnetBuildResult:
    path: Path
    file_bytes: int
    neuron_count: int
    connection_count: int
    sha256: str


@dataclass(frozen=True, slots=True)
class NbnetFileInfo:
    path: Path
    version: tuple[int, int]
    file_bytes: int
    metadata_bytes: int
    neuron_count: int
    connection_count: int
    checksum: str


@dataclass(frozen=True, slots=True)
class NbnetValidationReport:
    valid: bool
    info: NbnetFileInfo | None
    errors: tuple[str, ...]


# ------------------------------------------------------------------ parameters
def encode_parameter(value: Any) -> Any:
    """Kind-tagged JSON form of a parameter value (dicts recurse)."""
    if isinstance(value, NativeParameter):
        return {PARAMETER_MARKER: value.kind, "value": value.value}
    if isinstance(value, dict):
        return {str(k): encode_parameter(v) for k, v in value.items()}
    if isinstance(value, bool):
        kind = "bool"
    elif isinstance(value, int):
        kind = "int"
    elif isinstance(value, float):
        kind = "float"
    elif isinstance(value, str):
        kind = "str"
    elif isinstance(value, (list, tuple)):
        first = value[0] if value else 0
        kinds = {bool: "bool_list", int: "int_list", float: "float_list", str: "str_list"}
        kind = next((k for t, k in kinds.items() if type(first) is t), None)
        if kind is None:
            raise TypeError(f"unsupported nbnet parameter list item: {type(first).__name__}")
        value = list(value)
    else:
        raise TypeError(f"unsupported nbnet parameter value: {type(value).__name__}")
    return {PARAMETER_MARKER: kind, "value": value}


def decode_parameter(value: Any) -> Any:
    if isinstance(value, dict) and PARAMETER_MARKER in value:
        kind = value[PARAMETER_MARKER]
        payload = value.get("value")
        return NativeParameter(kind, payload) if kind in _NATIVE_KINDS else payload
    if isinstance(value, dict):
        return {k: decode_parameter(v) for k, v in value.items()}
    return value


def _object_metadata(obj) -> dict:
    d = obj.to_dict()
    d["parameters"] = encode_parameter(obj.parameters)
    return d


# --------------------------------------------------------------------- writer
def _column(value, count: int, dtype, name: str) -> np.ndarray:
    a = np.asarray(value)
    if a.ndim == 0:
        return np.full(count, a, dtype=dtype)
    a = a.ravel()
    if len(a) == 1:
        return np.full(count, a[0], dtype=dtype)
    if len(a) != count:
        raise ValueError(f"{name} length must be 1 or {count}, got {len(a)}")
    return a


class NbnetDescriptionBuilder:
    """Incrementally author a ``.nbnet`` file; connection batches are spooled
    to disk as they arrive, so the builder never holds the whole graph."""

    def __init__(self, path, *, options: NbnetWriteOptions | None = None):
        self.path = Path(path)
        self.options = options or NbnetWriteOptions()
        self._metadata = {"layers": [], "learning_rules": [], "outer_dynamics": [],
                          "outer_dynamic_connections": [], "input_convs": []}
        self._neuron_count = 0
        self._connection_count = 0
        self._result: NbnetBuildResult | None = None
        self._closed = False
        self.path.parent.mkdir(parents=True, exist_ok=True)
        self._spool = tempfile.NamedTemporaryFile(mode="w+b", prefix=f".{self.path.name}.",
                                                  suffix=".records.tmp", dir=self.path.parent, delete=False)
        self._spool_path = Path(self._spool.name)

    @property
    def result(self) -> NbnetBuildResult | None:
        return self._result

    def add_layer(self, layer: NeuronLayer) -> NbnetLayerHandle:
        self._ensure_open()
        if not isinstance(layer, NeuronLayer):
            raise TypeError("add_layer expects a NeuronLayer")
        if self._connection_count:
            raise RuntimeError("all layers must be added before the first connection batch")
        handle = NbnetLayerHandle(len(self._metadata["layers"]), self._neuron_count, layer.count)
        self._metadata["layers"].append(_object_metadata(layer))
        self._neuron_count += layer.count
        return handle

    def add_learning_rule(self, rule: LearningRule) -> int:
        self._ensure_open()
        if not isinstance(rule, LearningRule):
            raise TypeError("add_learning_rule expects a LearningRule")
        self._metadata["learning_rules"].append(_object_metadata(rule))
        return len(self._metadata["learning_rules"]) - 1

    def append_connections(self, source, target, *, synapse_type=0, weight=1.0, max_weight=None, delay=1,
                           synapse_rule=-1, trigger_rule=-1) -> int:
        """Append one batch (scalars broadcast) without retaining it."""
        self._ensure_open()
        if not self._metadata["layers"]:
            raise RuntimeError("at least one layer must be added before connections")
        src = np.asarray(source, dtype=np.int64).ravel()
        dst = np.asarray(target, dtype=np.int64).ravel()
        count = len(src)
        if len(dst) != count:
            raise ValueError("source and target lengths must match")
        w = _column(weight, count, np.float64, "weight")
        wmax = w if max_weight is None else _column(max_weight, count, np.float64, "max_weight")
        cols = {"synapse_type": _column(synapse_type, count, np.int64, "synapse_type"),
                "delay": _column(delay, count, np.int64, "delay"),
                "synapse_rule": _column(synapse_rule, count, np.int64, "synapse_rule"),
                "trigger_rule": _column(trigger_rule, count, np.int64, "trigger_rule")}
        if count:
            if src.min() < 0 or dst.min() < 0 or cols["delay"].min() < 0:
                raise ValueError("source, target, and delay must be non-negative")
            if src.max() >= self._neuron_count or dst.max() >= self._neuron_count:
                bad = int(np.flatnonzero((src >= self._neuron_count) | (dst >= self._neuron_count))[0])
                raise ValueError(f"connection neuron id is out of range [0, {self._neuron_count}): "
                                 f"{int(src[bad])} -> {int(dst[bad])}")
            if cols["delay"].max() > 0xFFFFFFFF:
                raise ValueError("delay exceeds the nbnet v1 uint32 range")
            lim = (-(2 ** 31), 2 ** 31 - 1)
            if cols["synapse_type"].min() < lim[0] or cols["synapse_type"].max() > lim[1]:
                raise ValueError("synapse_type exceeds the nbnet v1 int32 range")
            for k in ("synapse_rule", "trigger_rule"):
                if cols[k].min() < lim[0] or cols[k].max() > lim[1]:
                    raise ValueError("learning-rule index exceeds the nbnet v1 int32 range")
            if not (np.all(np.isfinite(w)) and np.all(np.isfinite(wmax))):
                raise ValueError("weight and max_weight must be finite")
        rec = np.empty(count, RECORD)
        rec["source"], rec["target"] = src, dst
        rec["synapse_type"] = cols["synapse_type"]
        rec["weight"], rec["max_weight"] = w, wmax
        rec["delay"] = cols["delay"]
        rec["synapse_rule"], rec["trigger_rule"] = cols["synapse_rule"], cols["trigger_rule"]
        self._spool.write(rec.tobytes())
        self._connection_count += count
        return count

    def append_connection(self, connection: Connection) -> int:
        if not isinstance(connection, Connection):
            raise TypeError("append_connection expects a Connection")
        return self.append_connections(**connection.normalized())

    def finalize(self) -> NbnetBuildResult:
        if self._result is not None:
            return self._result
        self._ensure_open()
        if self.path.exists() and not self.options.overwrite:
            raise FileExistsError(f"refusing to overwrite existing nbnet file: {self.path}")
        metadata = json.dumps(self._metadata, ensure_ascii=False, sort_keys=True,
                              separators=(",", ":")).encode("utf-8")
        digest = hashlib.sha256(metadata)
        self._spool.flush()
        self._spool.seek(0)
        tmp = self.path.with_name(f".{self.path.name}.{os.getpid()}.tmp")
        try:
            with tmp.open("w+b") as out:
                out.write(b"\0" * HEADER.size)
                out.write(metadata)
                while chunk := self._spool.read(1 << 20):
                    out.write(chunk)
                    digest.update(chunk)
                out.seek(0)
                out.write(HEADER.pack(MAGIC, VERSION_MAJOR, VERSION_MINOR, FLAG_SHA256, RECORD.itemsize,
                                      len(metadata), self._connection_count, digest.digest()))
                out.flush()
                if self.options.fsync:
                    os.fsync(out.fileno())
            os.replace(tmp, self.path)
        finally:
            if tmp.exists():
                tmp.unlink()
            self._close_spool()
        self._result = NbnetBuildResult(self.path.resolve(), self.path.stat().st_size, self._neuron_count,
                                        self._connection_count, digest.hexdigest())
        return self._result

    def abort(self) -> None:
        self._close_spool()

    def _ensure_open(self) -> None:
        if self._closed:
            raise RuntimeError("nbnet builder is closed")

    def _close_spool(self) -> None:
        if self._closed:
            return
        self._closed = True
        self._spool.close()
        if self._spool_path.exists():
            self._spool_path.unlink()

    def __enter__(self) -> "NbnetDescriptionBuilder":
        return self

    def __exit__(self, exc_type, exc, tb) -> None:
        if exc_type is None and self._result is None:
            self.finalize()
        else:
            self._close_spool()


def from_network(network: Network, path, *, options: NbnetWriteOptions | None = None) -> NbnetBuildResult:
    """Write an in-memory ``Network`` as ``.nbnet``."""
    if not isinstance(network, Network):
        raise TypeError("from_network expects a neuronbridge_gb300.Network")
    builder = NbnetDescriptionBuilder(path, options=options)
    try:
        for layer in network.layers:
            builder.add_layer(layer)
        for rule in network.learning_rules:
            builder.add_learning_rule(rule)
        for connection in network.connections:
            builder.append_connection(connection)
        return builder.finalize()
    except BaseException:
        builder.abort()
        raise


def from_batches(path, layers: Iterable[NeuronLayer], connection_batches: Iterable[Mapping[str, Any]], *,
                 learning_rules: Iterable[LearningRule] = (),
                 options: NbnetWriteOptions | None = None) -> NbnetBuildResult:
    """Write ``.nbnet`` straight from an iterable of connection batches."""
    builder = NbnetDescriptionBuilder(path, options=options)
    try:
        for layer in layers:
            builder.add_layer(layer)
        for rule in learning_rules:
            builder.add_learning_rule(rule)
        for batch in connection_batches:
            builder.append_connections(**dict(batch))
        return builder.finalize()
    except BaseException:
        builder.abort()
        raise


# --------------------------------------------------------------------- reader
def _read_file(path, *, verify_checksum: bool) -> tuple[Path, dict, NbnetFileInfo]:
    file_path = Path(path)
    file_bytes = file_path.stat().st_size
    with file_path.open("rb") as stream:
        raw = stream.read(HEADER.size)
        if len(raw) != HEADER.size:
            raise ValueError("truncated nbnet header")
        magic, major, minor, flags, record_size, metadata_size, count, expected = HEADER.unpack(raw)
        if magic != MAGIC:
            raise ValueError("invalid nbnet magic")
        if major != VERSION_MAJOR:
            raise ValueError(f"unsupported nbnet major version: {major}")
        if record_size != RECORD.itemsize:
            raise ValueError(f"unsupported connection record size: {record_size}")
        if metadata_size > MAX_METADATA_BYTES:
            raise ValueError(f"nbnet metadata exceeds {MAX_METADATA_BYTES} bytes")
        expected_size = HEADER.size + metadata_size + count * record_size
        if file_bytes != expected_size:
            raise ValueError(f"nbnet size mismatch: expected {expected_size}, got {file_bytes}")
        metadata_bytes = stream.read(metadata_size)
        if len(metadata_bytes) != metadata_size:
            raise ValueError("truncated nbnet metadata")
        if verify_checksum:
            if not flags & FLAG_SHA256:
                raise ValueError("nbnet file does not contain a supported checksum")
            digest = hashlib.sha256(metadata_bytes)
            while chunk := stream.read(1 << 20):
                digest.update(chunk)
            if digest.digest() != expected:
                raise ValueError("nbnet checksum mismatch")
    metadata = json.loads(metadata_bytes.decode("utf-8"))
    if not isinstance(metadata, dict) or not isinstance(metadata.get("layers", []), list):
        raise ValueError("nbnet metadata must contain a layers list")
    try:
        neurons = sum(int(layer["count"]) for layer in metadata.get("layers", []))
    except (KeyError, TypeError, ValueError) as exc:
        raise ValueError("invalid nbnet layer metadata") from exc
    info = NbnetFileInfo(file_path.resolve(), (major, minor), file_bytes, metadata_size, neurons, count,
                         expected.hex())
    return file_path, metadata, info


def inspect(path, *, verify_checksum: bool = False) -> NbnetFileInfo:
    return _read_file(path, verify_checksum=verify_checksum)[2]


def validate(path, *, verify_checksum: bool = True) -> NbnetValidationReport:
    try:
        return NbnetValidationReport(True, inspect(path, verify_checksum=verify_checksum), ())
    except (OSError, ValueError, TypeError, KeyError, UnicodeDecodeError, struct.error) as exc:
        return NbnetValidationReport(False, None, (str(exc),))


def is_valid(path, *, verify_checksum: bool = True) -> bool:
    return validate(path, verify_checksum=verify_checksum).valid


def load(path, options: StreamingBuildOptions | None = None) -> tuple[NetworkDescription, dict]:
    """Read a ``.nbnet`` file into the engine's flat description, streaming
    the connection records in batches of at most the memory budget."""
    options = options or StreamingBuildOptions()
    started = time.perf_counter()
    file_path, meta, info = _read_file(path, verify_checksum=options.verify_checksum)
    for key in ("outer_dynamics", "outer_dynamic_connections", "input_convs"):
        if meta.get(key):
            raise ValueError(f"nbnet {key} are not supported by the GB300 engine")
    layers = []
    for entry in meta["layers"]:
        params = decode_parameter(entry.get("parameters", {}))
        layers.append(NeuronLayer(entry["model"], int(entry["count"]),
                                  update_timestep=int(entry.get("update_timestep", 1)),
                                  monitored=bool(entry.get("monitored", False)),
                                  output=bool(entry.get("output", False)),
                                  communication_input=bool(entry.get("communication_input", False)),
                                  parameters=params))
    rules = [LearningRule(r["name"], decode_parameter(r.get("parameters", {})))
             for r in meta.get("learning_rules", [])]
    desc = NetworkDescription(layers, [], rules)
    n = info.connection_count
    cols = {"source": np.empty(n, np.int32), "target": np.empty(n, np.int32), "type": np.empty(n, np.int32),
            "weight": np.empty(n, np.float32), "max_weight": np.empty(n, np.float32),
            "delay": np.empty(n, np.int32), "rule": np.empty(n, np.int32)}
    batch = max(1, (options.memory_budget_mb << 20) // RECORD.itemsize)
    offset = HEADER.size + info.metadata_bytes
    neurons = info.neuron_count
    if n:
        if options.mmap:
            records = np.memmap(file_path, dtype=RECORD, mode="r", offset=offset, shape=(n,))
            read = lambda a, b: records[a:b]
        else:
            fh = file_path.open("rb")
            read = lambda a, b: (fh.seek(offset + a * RECORD.itemsize),
                                 np.frombuffer(fh.read((b - a) * RECORD.itemsize), RECORD))[1]
        try:
            for a in range(0, n, batch):
                b = min(n, a + batch)
                r = read(a, b)
                if r["source"].max() >= neurons or r["target"].max() >= neurons:
                    raise ValueError(f"nbnet connection neuron id is out of range [0, {neurons})")
                if np.any(r["trigger_rule"] != -1):
                    raise ValueError("trigger rules are not supported by the GB300 engine")
                if r["delay"].max() > 0x7FFFFFFF:
                    raise ValueError("nbnet delay exceeds the engine's range")
                cols["source"][a:b] = r["source"]
                cols["target"][a:b] = r["target"]
                cols["type"][a:b] = r["synapse_type"]
                cols["weight"][a:b] = r["weight"]
                cols["max_weight"][a:b] = r["max_weight"]
                cols["delay"][a:b] = r["delay"]
                cols["rule"][a:b] = r["synapse_rule"]
        finally:
            if not options.mmap:
                fh.close()
            else:
                del records
    for k, v in cols.items():
        setattr(desc, k, v)
    stats = {"mode": "streaming", "path": str(file_path), "file_bytes": info.file_bytes,
             "metadata_bytes": info.metadata_bytes, "neuron_count": neurons, "connection_count": n,
             "batch_records": int(min(batch, n)) if n else 0, "memory_budget_bytes": options.memory_budget_mb << 20,
             "mmap": bool(options.mmap), "checksum_verified": bool(options.verify_checksum),
             "description_load_seconds": time.perf_counter() - started, "runtime_build_path": "streaming_direct"}
    return desc, stats


__all__ = ["NbnetBuildResult", "NbnetDescriptionBuilder", "NbnetFileInfo", "NbnetLayerHandle",
           "NbnetValidationReport", "NbnetWriteOptions", "StreamingBuildOptions", "from_batches", "from_network",
           "inspect", "is_valid", "load", "validate"]
