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

Writing encodes each connection batch as one numpy record array and writes
it to an anonymous temporary file; ``finalize`` hashes metadata and records
while it writes the file beside its destination and renames it into place.
Loading reads the record block in slices bounded by the memory budget into
the engine's flat int32/float32 connection columns, so no per-connection
Python object is ever made; the engine then builds its CSC directly from
those columns.
"""
from __future__ import annotations

import hashlib
import json
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


# ------------------------------------------------------------------ header
@dataclass(frozen=True, slots=True)
class _Header:
    """The fixed-size file header and the checks a reader makes on it."""

    flags: int
    metadata_size: int
    count: int
    digest: bytes
    version: tuple[int, int] = (VERSION_MAJOR, VERSION_MINOR)

    def pack(self) -> bytes:
        return HEADER.pack(MAGIC, self.version[0], self.version[1], self.flags, RECORD.itemsize,
                           self.metadata_size, self.count, self.digest)

    @classmethod
    def parse(cls, raw: bytes, file_bytes: int) -> "_Header":
        if len(raw) != HEADER.size:
            raise ValueError("truncated nbnet header")
        magic, major, minor, flags, record_size, metadata_size, count, digest = HEADER.unpack(raw)
        if magic != MAGIC:
            raise ValueError("invalid nbnet magic")
        if major != VERSION_MAJOR:
            raise ValueError(f"unsupported nbnet major version: {major}")
        if record_size != RECORD.itemsize:
            raise ValueError(f"unsupported connection record size: {record_size}")
        if metadata_size > MAX_METADATA_BYTES:
            raise ValueError(f"nbnet metadata exceeds {MAX_METADATA_BYTES} bytes")
        size = HEADER.size + metadata_size + count * RECORD.itemsize
        if file_bytes != size:
            raise ValueError(f"nbnet size mismatch: expected {size}, got {file_bytes}")
        return cls(flags, metadata_size, count, digest, (major, minor))

    @property
    def records_offset(self) -> int:
        return HEADER.size + self.metadata_size


# ----------------------------------------------------------------- records
_INT32 = (-(2 ** 31), 2 ** 31 - 1)


def _broadcast(value, count: int, dtype, name: str) -> np.ndarray:
    """A connection column: a scalar or length-1 value repeated, or exactly
    `count` values."""
    a = np.asarray(value).ravel()
    if a.size == 1:
        return np.full(count, a[0], dtype=dtype)
    if a.size != count:
        raise ValueError(f"{name} length must be 1 or {count}, got {a.size}")
    return a.astype(dtype, copy=False)


def _encode_batch(neurons: int, source, target, synapse_type, weight, max_weight, delay, synapse_rule,
                  trigger_rule) -> np.ndarray:
    """One batch of connections as an array of 32-byte records, every value
    checked against the file's field ranges first."""
    src = np.asarray(source, dtype=np.int64).ravel()
    dst = np.asarray(target, dtype=np.int64).ravel()
    n = src.size
    if dst.size != n:
        raise ValueError("source and target lengths must match")
    w = _broadcast(weight, n, np.float64, "weight")
    wmax = w if max_weight is None else _broadcast(max_weight, n, np.float64, "max_weight")
    ints = {k: _broadcast(v, n, np.int64, k) for k, v in
            (("synapse_type", synapse_type), ("delay", delay), ("synapse_rule", synapse_rule),
             ("trigger_rule", trigger_rule))}
    out = np.empty(n, RECORD)
    if n == 0:
        return out
    if min(src.min(), dst.min(), ints["delay"].min()) < 0:
        raise ValueError("source, target, and delay must be non-negative")
    outside = (src >= neurons) | (dst >= neurons)
    if outside.any():
        k = int(np.argmax(outside))
        raise ValueError(f"connection neuron id is out of range [0, {neurons}): {int(src[k])} -> {int(dst[k])}")
    if ints["delay"].max() > 0xFFFFFFFF:
        raise ValueError("delay exceeds the nbnet v1 uint32 range")

    def in_int32(a):
        return _INT32[0] <= a.min() and a.max() <= _INT32[1]

    if not in_int32(ints["synapse_type"]):
        raise ValueError("synapse_type exceeds the nbnet v1 int32 range")
    if not (in_int32(ints["synapse_rule"]) and in_int32(ints["trigger_rule"])):
        raise ValueError("learning-rule index exceeds the nbnet v1 int32 range")
    if not (np.isfinite(w).all() and np.isfinite(wmax).all()):
        raise ValueError("weight and max_weight must be finite")
    out["source"], out["target"], out["weight"], out["max_weight"] = src, dst, w, wmax
    for k, v in ints.items():
        out[k] = v
    return out


class _RecordSink:
    """Connection records as they are appended, in an anonymous temporary
    file beside the destination (the operating system removes it when it is
    closed, whatever happens to the build)."""

    def __init__(self, directory: Path):
        self.file = tempfile.TemporaryFile(mode="w+b", dir=directory)
        self.count = 0

    def write(self, records: np.ndarray) -> None:
        self.file.write(records.tobytes())
        self.count += len(records)

    def chunks(self, size: int = 1 << 20):
        self.file.flush()
        self.file.seek(0)
        while chunk := self.file.read(size):
            yield chunk

    def close(self) -> None:
        self.file.close()


def _emit(path: Path, metadata: bytes, sink: _RecordSink, options: "NbnetWriteOptions") -> tuple[str, int]:
    """Write header, metadata and the sink's records to a temporary file in
    the destination directory, hashing as it goes, then move it into place
    in one rename.  Returns (hex digest, file size)."""
    fd, tmp_name = tempfile.mkstemp(prefix=f".{path.name}.", suffix=".tmp", dir=path.parent)
    tmp = Path(tmp_name)
    try:
        with os.fdopen(fd, "w+b") as out:
            digest = hashlib.sha256(metadata)
            out.seek(HEADER.size)
            out.write(metadata)
            for chunk in sink.chunks():
                out.write(chunk)
                digest.update(chunk)
            out.seek(0)
            out.write(_Header(FLAG_SHA256, len(metadata), sink.count, digest.digest()).pack())
            out.flush()
            if options.fsync:
                os.fsync(out.fileno())
        os.replace(tmp, path)
    finally:
        tmp.unlink(missing_ok=True)
    return digest.hexdigest(), path.stat().st_size


# ------------------------------------------------------------------ writer
class NbnetDescriptionBuilder:
    """Incremental ``.nbnet`` authoring.  Layers come first, then any number
    of connection batches (learning rules at any time); each batch is encoded
    and written out as it arrives, so memory does not grow with the network.
    ``finalize`` writes the file; ``abort`` (or leaving a ``with`` block on
    an exception) drops everything."""

    _OPEN, _DONE, _ABORTED = "open", "done", "aborted"

    def __init__(self, path, *, options: NbnetWriteOptions | None = None):
        self.path = Path(path)
        self.options = options or NbnetWriteOptions()
        self.path.parent.mkdir(parents=True, exist_ok=True)
        self._layers: list[dict] = []
        self._rules: list[dict] = []
        self._neurons = 0
        self._sink = _RecordSink(self.path.parent)
        self._state = self._OPEN
        self._result: NbnetBuildResult | None = None

    @property
    def result(self) -> NbnetBuildResult | None:
        return self._result

    def _require_open(self) -> None:
        if self._state != self._OPEN:
            raise RuntimeError("nbnet builder is closed")

    def add_layer(self, layer: NeuronLayer) -> NbnetLayerHandle:
        self._require_open()
        if not isinstance(layer, NeuronLayer):
            raise TypeError("add_layer expects a NeuronLayer")
        if self._sink.count:
            raise RuntimeError("all layers must be added before the first connection batch")
        handle = NbnetLayerHandle(len(self._layers), self._neurons, layer.count)
        self._layers.append(_tagged(layer))
        self._neurons += layer.count
        return handle

    def add_learning_rule(self, rule: LearningRule) -> int:
        self._require_open()
        if not isinstance(rule, LearningRule):
            raise TypeError("add_learning_rule expects a LearningRule")
        self._rules.append(_tagged(rule))
        return len(self._rules) - 1

    def append_connections(self, source, target, *, synapse_type=0, weight=1.0, max_weight=None, delay=1,
                           synapse_rule=-1, trigger_rule=-1) -> int:
        """Encode and write one batch (scalars broadcast); nothing is kept."""
        self._require_open()
        if not self._layers:
            raise RuntimeError("at least one layer must be added before connections")
        records = _encode_batch(self._neurons, source, target, synapse_type, weight, max_weight, delay,
                                synapse_rule, trigger_rule)
        self._sink.write(records)
        return len(records)

    def append_connection(self, connection: Connection) -> int:
        if not isinstance(connection, Connection):
            raise TypeError("append_connection expects a Connection")
        return self.append_connections(**connection.normalized())

    def finalize(self) -> NbnetBuildResult:
        if self._result is not None:
            return self._result
        self._require_open()
        if self.path.exists() and not self.options.overwrite:
            raise FileExistsError(f"refusing to overwrite existing nbnet file: {self.path}")
        metadata = {"layers": self._layers, "learning_rules": self._rules, "outer_dynamics": [],
                    "outer_dynamic_connections": [], "input_convs": []}
        blob = json.dumps(metadata, ensure_ascii=False, sort_keys=True, separators=(",", ":")).encode("utf-8")
        try:
            digest, size = _emit(self.path, blob, self._sink, self.options)
        finally:
            self._release(self._DONE)
        self._result = NbnetBuildResult(self.path.resolve(), size, self._neurons, self._sink.count, digest)
        return self._result

    def abort(self) -> None:
        self._release(self._ABORTED)

    def _release(self, state: str) -> None:
        if self._state == self._OPEN:
            self._sink.close()
            self._state = state

    def __enter__(self) -> "NbnetDescriptionBuilder":
        return self

    def __exit__(self, exc_type, exc, tb) -> None:
        if exc_type is not None:
            self.abort()
        elif self._result is None:
            self.finalize()


def _tagged(obj) -> dict:
    """Metadata entry of a layer or learning rule, parameters kind-tagged."""
    entry = obj.to_dict()
    entry["parameters"] = encode_parameter(obj.parameters)
    return entry


def _build(path, options, layers, rules, batches) -> NbnetBuildResult:
    with NbnetDescriptionBuilder(path, options=options) as builder:
        for layer in layers:
            builder.add_layer(layer)
        for rule in rules:
            builder.add_learning_rule(rule)
        for batch in batches:
            builder.append_connections(**batch)
        return builder.finalize()  # inside the block: a failure here aborts the build


def from_network(network: Network, path, *, options: NbnetWriteOptions | None = None) -> NbnetBuildResult:
    """Write an in-memory ``Network`` as ``.nbnet``."""
    if not isinstance(network, Network):
        raise TypeError("from_network expects a neuronbridge_gb300.Network")
    return _build(path, options, network.layers, network.learning_rules,
                  (c.normalized() for c in network.connections))


def from_batches(path, layers: Iterable[NeuronLayer], connection_batches: Iterable[Mapping[str, Any]], *,
                 learning_rules: Iterable[LearningRule] = (),
                 options: NbnetWriteOptions | None = None) -> NbnetBuildResult:
    """Write ``.nbnet`` straight from an iterable of connection batches."""
    return _build(path, options, layers, learning_rules, (dict(b) for b in connection_batches))


# ------------------------------------------------------------------ reader
@dataclass(frozen=True, slots=True)
class _Parsed:
    path: Path
    header: _Header
    metadata: dict
    info: NbnetFileInfo


def _parse(path, *, verify_checksum: bool) -> _Parsed:
    """Header, metadata and summary of a file, every structural check made
    (and the checksum over metadata and records when asked)."""
    file_path = Path(path)
    size = file_path.stat().st_size
    with file_path.open("rb") as f:
        header = _Header.parse(f.read(HEADER.size), size)
        blob = f.read(header.metadata_size)
        if len(blob) != header.metadata_size:
            raise ValueError("truncated nbnet metadata")
        if verify_checksum:
            if not header.flags & FLAG_SHA256:
                raise ValueError("nbnet file does not contain a supported checksum")
            digest = hashlib.sha256(blob)
            for chunk in iter(lambda: f.read(1 << 20), b""):
                digest.update(chunk)
            if digest.digest() != header.digest:
                raise ValueError("nbnet checksum mismatch")
    metadata = json.loads(blob.decode("utf-8"))
    if not isinstance(metadata, dict) or not isinstance(metadata.get("layers", []), list):
        raise ValueError("nbnet metadata must contain a layers list")
    try:
        neurons = sum(int(layer["count"]) for layer in metadata.get("layers", []))
    except (KeyError, TypeError, ValueError) as exc:
        raise ValueError("invalid nbnet layer metadata") from exc
    info = NbnetFileInfo(file_path.resolve(), header.version, size, header.metadata_size, neurons, header.count,
                         header.digest.hex())
    return _Parsed(file_path, header, metadata, info)


def inspect(path, *, verify_checksum: bool = False) -> NbnetFileInfo:
    return _parse(path, verify_checksum=verify_checksum).info


def validate(path, *, verify_checksum: bool = True) -> NbnetValidationReport:
    try:
        return NbnetValidationReport(True, inspect(path, verify_checksum=verify_checksum), ())
    except (OSError, ValueError, TypeError, KeyError, UnicodeDecodeError, struct.error) as exc:
        return NbnetValidationReport(False, None, (str(exc),))


def is_valid(path, *, verify_checksum: bool = True) -> bool:
    return validate(path, verify_checksum=verify_checksum).valid


def _layer_from(entry: dict) -> NeuronLayer:
    return NeuronLayer(entry["model"], int(entry["count"]), update_timestep=int(entry.get("update_timestep", 1)),
                       monitored=bool(entry.get("monitored", False)), output=bool(entry.get("output", False)),
                       communication_input=bool(entry.get("communication_input", False)),
                       parameters=decode_parameter(entry.get("parameters", {})))


# the description's connection columns and the record fields they come from
_COLUMNS = (("source", "source", np.int32), ("target", "target", np.int32), ("type", "synapse_type", np.int32),
            ("weight", "weight", np.float32), ("max_weight", "max_weight", np.float32),
            ("delay", "delay", np.int32), ("rule", "synapse_rule", np.int32))


def load(path, options: StreamingBuildOptions | None = None) -> tuple[NetworkDescription, dict]:
    """Read a ``.nbnet`` file into the engine's flat description: the record
    block is read (mapped, or read with ``numpy.fromfile``) in slices of at
    most the memory budget, each checked and copied into preallocated
    int32 / float32 columns."""
    options = options or StreamingBuildOptions()
    started = time.perf_counter()
    parsed = _parse(path, verify_checksum=options.verify_checksum)
    meta, info = parsed.metadata, parsed.info
    for key in ("outer_dynamics", "outer_dynamic_connections", "input_convs"):
        if meta.get(key):
            raise ValueError(f"nbnet {key} are not supported by the GB300 engine")
    rules = [LearningRule(r["name"], decode_parameter(r.get("parameters", {})))
             for r in meta.get("learning_rules", [])]
    desc = NetworkDescription([_layer_from(e) for e in meta["layers"]], [], rules)
    n, neurons = info.connection_count, info.neuron_count
    cols = {name: np.empty(n, dtype) for name, _, dtype in _COLUMNS}
    step = max(1, (options.memory_budget_mb << 20) // RECORD.itemsize)
    offset = parsed.header.records_offset
    mapped = np.memmap(parsed.path, dtype=RECORD, mode="r", offset=offset, shape=(n,)) if (n and options.mmap) \
        else None
    try:
        for a in range(0, n, step):
            b = min(n, a + step)
            if mapped is not None:
                r = mapped[a:b]
            else:
                r = np.fromfile(parsed.path, dtype=RECORD, count=b - a, offset=offset + a * RECORD.itemsize)
            if r["source"].max() >= neurons or r["target"].max() >= neurons:
                raise ValueError(f"nbnet connection neuron id is out of range [0, {neurons})")
            if (r["trigger_rule"] != -1).any():
                raise ValueError("trigger rules are not supported by the GB300 engine")
            if r["delay"].max() > 0x7FFFFFFF:
                raise ValueError("nbnet delay exceeds the engine's range")
            for name, field, _ in _COLUMNS:
                cols[name][a:b] = r[field]
    finally:
        del mapped
    for name, values in cols.items():
        setattr(desc, name, values)
    stats = {"mode": "streaming", "path": str(parsed.path), "file_bytes": info.file_bytes,
             "metadata_bytes": info.metadata_bytes, "neuron_count": neurons, "connection_count": n,
             "batch_records": int(min(step, n)) if n else 0, "memory_budget_bytes": options.memory_budget_mb << 20,
             "mmap": bool(options.mmap), "checksum_verified": bool(options.verify_checksum),
             "description_load_seconds": time.perf_counter() - started, "runtime_build_path": "streaming_direct"}
    return desc, stats


__all__ = ["NbnetBuildResult", "NbnetDescriptionBuilder", "NbnetFileInfo", "NbnetLayerHandle",
           "NbnetValidationReport", "NbnetWriteOptions", "StreamingBuildOptions", "from_batches", "from_network",
           "inspect", "is_valid", "load", "validate"]
