"""Shared set-up of the STDP pin (tests/test_oracle_ref_stdp.py on the CPU,
tests/test_gpu_ref_stdp.py on the GPU): one golden case of
tests/golden/stdp_reference.json as a network and its external spikes.

Connection k is a plastic synapse from input-spike neuron k to one
voltage-jump LIF target, of type 1 (the reference subtracts type-1 weights,
so these arrivals never make the target fire) with the case's delay, weight
and maximum.  A pre event of connection k at tick t is a spike of neuron k at
t - delay[k].  A further input-spike neuron (the forcer) reaches the target
over a static weight of 1,000 with delay 1: a forcer spike at t - 1 makes
the target fire in the update of tick t, so the post events are exactly the
case's post ticks (at least two apart, since a spike at t gates the
arrivals of t + 1 with t_ref = 0)."""
from __future__ import annotations

import json
import os

import numpy as np

from neuronbridge_gb300 import Connection, LearningRule, Network, NeuronLayer, float32, int32

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "stdp_reference.json")


def load_cases() -> list[dict]:
    return json.load(open(GOLDEN))["cases"]


def network(case: dict) -> tuple[Network, np.ndarray, np.ndarray]:
    """(network, external spike times, their neuron ids)."""
    n = len(case["w0"])
    a_plus, tau_plus, a_minus, tau_minus = case["params"]
    net = Network()
    net.add_layer(NeuronLayer.input_spike(n))
    net.add_layer(NeuronLayer.input_spike(1))
    net.add_layer(NeuronLayer("TimeDrivenLIF_Voltage_jump", 1, output=True,
                              parameters={"V_rest": float32(-65.0), "V_reset": float32(-65.0),
                                          "V_th": float32(-50.0), "tau": float32(20.0), "R": float32(1.0),
                                          "t_ref": int32(0)}))
    net.add_learning_rule(LearningRule("STDP", {"Max_LTP": float32(a_plus), "LTP_tau": float32(tau_plus),
                                                "Max_LTD": float32(a_minus), "LTD_tau": float32(tau_minus)}))
    k = np.arange(n, dtype=np.int32)
    net.connect(Connection(k, np.full(n, n + 1, np.int32), synapse_type=1,
                           weight=np.asarray(case["w0"], np.float32), max_weight=np.asarray(case["wmax"], np.float32),
                           delay=np.asarray(case["delay"], np.int32), synapse_rule=0))
    net.connect(Connection(n, n + 1, synapse_type=0, weight=1000.0, delay=1))
    times, ids = [], []
    for c, ticks in enumerate(case["pre"]):
        times += [t - case["delay"][c] for t in ticks]
        ids += [c] * len(ticks)
    times += [t - 1 for t in case["post"]]
    ids += [n] * len(case["post"])
    return net, np.asarray(times, np.int64), np.asarray(ids, np.int64)
