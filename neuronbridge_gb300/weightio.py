"""Weight snapshots in the reference's format.

``NPGR_WEIGHT_SNAPSHOT 1`` (reference src/native/gpu/src/simulation_dense/
SimulationWeightIO.cpp:115-373): a header with the current time step, one
``block main 0 <count>`` of run-length-encoded weights in original connection
order (runs of exactly equal values, weights printed with 9 significant
digits so every float round-trips), optional ``block dense`` blocks, and
``end``.  Reading validates the structure with the reference's error texts.
"""
from __future__ import annotations

import re

import numpy as np

# whitespace-separated tokens, with a double-quoted name (std::quoted) as one
_TOKEN = re.compile(r'"(?:[^"\\]|\\.)*"|\S+')


def _rle_lines(weights: np.ndarray) -> list[str]:
    w = np.asarray(weights, np.float32)
    if w.size == 0:
        return []
    change = np.flatnonzero(w[1:] != w[:-1]) + 1
    starts = np.concatenate(([0], change))
    ends = np.concatenate((change, [w.size]))
    return [f"{e - s} {float(w[s]):.9g}" for s, e in zip(starts, ends)]


def write_snapshot(path, main_weights: np.ndarray, time_step: int, dense_blocks=()) -> None:
    """Write a snapshot (SimulationWeightIO.cpp:178-203); ``dense_blocks`` is
    a sequence of (name, weights)."""
    lines = ["NPGR_WEIGHT_SNAPSHOT 1", f"time_step {int(time_step)}", "",
             f"block main 0 {len(main_weights)}", "rle", *_rle_lines(main_weights), "end_block", ""]
    for index, (name, weights) in enumerate(dense_blocks):
        quoted = '"' + name.replace("\\", "\\\\").replace('"', '\\"') + '"'
        lines += [f"block dense {index} {quoted} {len(weights)}", "rle", *_rle_lines(weights), "end_block", ""]
    lines.append("end")
    try:
        with open(path, "w") as f:
            f.write("\n".join(lines) + "\n")
    except OSError:
        raise ValueError("failed to open weight snapshot for writing") from None


def _read_rle(tokens, pos: int, count: int):
    out = np.empty(count, np.float32)
    filled = 0
    while pos < len(tokens):
        tok = tokens[pos]
        if tok == "end_block":
            if filled != count:
                raise ValueError("RLE block ended with an unexpected weight count")
            return out, pos + 1
        run = _int(tok)
        if run is None:
            raise ValueError("RLE block contains an invalid run count")
        try:
            value = np.float32(float(tokens[pos + 1]))
        except (IndexError, ValueError):
            raise ValueError("RLE block is missing a weight value") from None
        if run <= 0:
            raise ValueError("RLE block contains a non-positive run count")
        if filled + run > count:
            raise ValueError("RLE block expands beyond its declared weight count")
        out[filled:filled + run] = value
        filled += run
        pos += 2
    raise ValueError("RLE block reached end-of-file before end_block")


def _int(tok):
    try:
        return int(tok)
    except (TypeError, ValueError):
        return None


def read_snapshot(path) -> dict:
    """Parse a snapshot; raise ValueError with the reference's reason text
    (SimulationWeightIO.cpp:205-275) on any structural fault."""
    try:
        tokens = _TOKEN.findall(open(path).read())
    except OSError:
        raise ValueError("failed to open weight snapshot for reading") from None
    at = lambda i: tokens[i] if i < len(tokens) else None
    if at(0) != "NPGR_WEIGHT_SNAPSHOT" or _int(at(1)) != 1:
        raise ValueError("weight file is not an NPGR_WEIGHT_SNAPSHOT v1 file")
    if at(2) != "time_step" or _int(at(3)) is None:
        raise ValueError("weight snapshot is missing time_step")
    snap = {"time_step": _int(at(3)), "main": None, "dense": []}
    pos = 4
    while pos < len(tokens):
        tok = tokens[pos]
        if tok == "end":
            if snap["main"] is None:
                raise ValueError("weight snapshot is missing main block")
            return snap
        if tok != "block":
            raise ValueError("weight snapshot contains an unexpected token")
        kind = at(pos + 1)
        if kind is None:
            raise ValueError("weight snapshot block is missing a kind")
        if kind == "main":
            index, count = _int(at(pos + 2)), _int(at(pos + 3))
            if index != 0 or count is None or count < 0:
                raise ValueError("main weight block header is invalid")
            if snap["main"] is not None:
                raise ValueError("weight snapshot contains duplicate main blocks")
            if at(pos + 4) != "rle":
                raise ValueError("main weight block is missing rle marker")
            snap["main"], pos = _read_rle(tokens, pos + 5, count)
        elif kind == "dense":
            index, name, count = _int(at(pos + 2)), at(pos + 3), _int(at(pos + 4))
            if index is None or name is None or count is None or count < 0:
                raise ValueError("dense weight block header is invalid")
            if at(pos + 5) != "rle":
                raise ValueError("dense weight block is missing rle marker")
            weights, pos = _read_rle(tokens, pos + 6, count)
            if len(name) >= 2 and name[0] == name[-1] == '"':
                name = re.sub(r'\\(.)', r'\1', name[1:-1])
            snap["dense"].append((index, name, weights))
        else:
            raise ValueError("weight snapshot contains an unknown block kind")
    raise ValueError("weight snapshot reached end-of-file before end marker")
