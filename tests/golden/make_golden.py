"""Generate golden known-answer vectors from the reference's own KAT script.

Run it in a checkout that has a copy of the reference project (read-only),
giving the reference's root directory as the one argument:

    python tests/golden/make_golden.py <reference-root>

It never executes the reference script's module-level code (that code builds
a Windows results directory and needs the compiled ``neuronbridge._core``).
Instead it parses ``numerical_accuracy_tests.py`` with ``ast``, keeps the
constant assignments and function definitions, and runs the expected-value
half of each test against a stand-in ``neuronbridge`` module whose
``Simulation`` returns the documented initial state:

* ``test_lif_voltage_jump``: the initial voltage read from the simulation is
  V_reset + random_mu = -5.0 for the parameters the test passes
  (reference: src/native/legacy/source_file_realtime_v1_async/NeuralModel/
  src/TimeDriven/TimeDrivenLIF_Voltage_jump.cpp:37, random_mu defaults to 0).
* ``test_izhikevich``: the float32 restatement that the reference reports as
  matching its native trajectory with max error 0
  (numerical_accuracy_report.md, "TimeDrivenIzhikevic_Exponential_Decay | 0").
* ``test_poisson``: the PoissonRate hash spike sequence.

Output: tests/golden/numerical_accuracy_kat.json (committed).
"""
from __future__ import annotations

import ast
import json
import os
import sys
import types

HERE = os.path.dirname(os.path.abspath(__file__))


class _FakeSim:
    def __init__(self, *args, **kwargs):
        pass

    def init(self):
        return self

    def add_external_currents(self, *args):
        return self

    def run(self, *args):
        return self

    def neuron_state(self, neuron_id):
        # documented initial state of the voltage-jump LIF (V_reset=-5 + mu=0)
        return {"state_variables": [-5.0, 0.0, 0.0, 0.0, 0.0, 0.0]}

    def output_spikes(self):
        return []


def _fake_neuronbridge():
    nb = types.ModuleType("neuronbridge")

    class _Layer:
        def __init__(self, *a, **k):
            pass

        @classmethod
        def input_current(cls, *a, **k):
            return cls()

    class _Net:
        def add_layer(self, *a):
            return self

        def connect(self, *a):
            return self

    nb.Network = _Net
    nb.NeuronLayer = _Layer
    nb.Connection = lambda *a, **k: None
    nb.Simulation = _FakeSim
    nb.SimulationConfig = lambda *a, **k: None
    nb.float32 = float
    return nb


def main(reference_root: str) -> None:
    path = os.path.join(reference_root, "numerical_accuracy_tests.py")
    tree = ast.parse(open(path, encoding="utf-8").read(), filename=path)
    keep = []
    for node in tree.body:
        if isinstance(node, ast.FunctionDef):
            keep.append(node)
        elif isinstance(node, ast.Assign) and all(isinstance(t, ast.Name) for t in node.targets):
            names = {t.id for t in node.targets}
            if names <= {"DT", "STEPS", "CURRENT", "TOL", "INTERNAL_SUBSTEPS_PER_RUN"}:
                keep.append(node)
        elif isinstance(node, (ast.Import, ast.ImportFrom)):
            keep.append(node)
    module = ast.Module(body=keep, type_ignores=[])
    sys.modules["neuronbridge"] = _fake_neuronbridge()
    ns: dict = {"__name__": "reference_kat"}
    exec(compile(module, path, "exec"), ns)

    lif = ns["test_lif_voltage_jump"]()
    izh = ns["test_izhikevich"]()
    poi = ns["test_poisson"]()
    out = {
        "source": "numerical_accuracy_tests.py (reference), expected-value functions only",
        "timestep": ns["DT"],
        "steps": ns["STEPS"],
        "current": ns["CURRENT"],
        "tolerance": ns["TOL"],
        "internal_substeps_first_run": ns["INTERNAL_SUBSTEPS_PER_RUN"],
        "lif_voltage_jump": {
            "parameters": {"V_rest": 0.0, "V_reset": -5.0, "V_th": 20.0, "tau": 10.0, "R": 1.0},
            "initial_voltage": lif["initial_voltage"],
            "expected_v": lif["expected"],
        },
        "izhikevich": {
            "expected_v": izh["voltage"]["expected"],
            "expected_u": izh["recovery"]["expected"],
            "first_state_report": {"V": -65.03999328613281, "U": -13.01200008392334},
        },
        "poisson": {
            "rate_bias_hz": 40.0,
            "timestep": 1.0,
            "steps": 200,
            "expected_spikes": [list(p) for p in poi["expected"]],
        },
    }
    dst = os.path.join(HERE, "numerical_accuracy_kat.json")
    with open(dst, "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", dst)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <reference-root>")
    main(sys.argv[1])
