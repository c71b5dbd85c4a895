"""Seeded synthetic networks for the benchmark and parity configurations.

The reference publishes no benchmark dataset; every input here is synthetic
and seeded (numpy ``default_rng``, PCG64).  Each builder returns a
:class:`~neuronbridge_gb300.model.Network` plus the ``SimulationConfig`` it is
run with, and takes a ``scale`` (or size) argument so that tests can run the
same construction at sizes the CPU oracle finishes in seconds.

* ``plain_lif``         1,000 voltage-jump LIF (800 E / 200 I), ER p=0.1,
                        w_E=+0.5 mV, w_I=-2.5 mV (type-1 weight 2.5), delay
                        15 steps, 1:1 PoissonRate drive at 8 kHz (+0.5 mV,
                        delay 1), dt=0.1 ms, 10,000 steps.
* ``izhikevich_stdp``   100k current-based Izhikevich (80k RS, 20k FS), RK4,
                        fixed in-degree 100 (sources uniform, self excluded,
                        drawn with replacement), delays 1..20 ms, w_E=6 with
                        pair STDP (A+=0.1, A-=0.12, tau=20 ms, clip [0,10]),
                        w_I=-5 (type-1 weight 5), dt=0.1 ms.  Noise: the
                        N(0, 5^2) current of Izhikevich (2003) is drawn once
                        per millisecond there; at dt = 0.1 ms a per-step
                        current with sigma = 5*sqrt(1 ms/dt) = 15.81 has the
                        same integrated effect per millisecond (sigma = 5 per
                        0.1-ms step leaves the network silent).
* ``batched_lif``       256 plain-LIF instances, sizes log-uniform in
                        [500, 50000], in-degree ~100, Poisson drive at
                        4..12 kHz, run as one network of disjoint instances.
"""
from __future__ import annotations

import numpy as np

from .model import (Connection, LearningRule, Network, NetworkDescription, NeuronLayer, SimulationConfig, float32,
                    int32)

LIF_PARAMS = {"V_rest": float32(-65.0), "V_reset": float32(-65.0), "V_th": float32(-50.0), "tau": float32(20.0),
              "R": float32(1.0), "t_ref": int32(20)}


def _lif_layer(count: int, output: bool = True) -> NeuronLayer:
    return NeuronLayer("TimeDrivenLIF_Voltage_jump", count, output=output, parameters=dict(LIF_PARAMS))


def plain_lif(n: int = 1000, steps: int = 10000, seed: int = 0, rate_hz: float = 8000.0, p: float = 0.1,
              delay: int = 15) -> tuple[Network, SimulationConfig]:
    """Configuration 0: plain LIF network with Poisson drive."""
    rng = np.random.default_rng(seed)
    n_exc = (n * 4) // 5
    net = Network()
    net.add_layer(_lif_layer(n))
    net.add_layer(NeuronLayer.poisson_rate(n, rate_bias_hz=rate_hz, rate_gain_hz_per_current=0.0))
    mask = rng.random((n, n)) < p
    np.fill_diagonal(mask, False)
    src, tgt = np.nonzero(mask)
    exc = src < n_exc
    net.connect(Connection(src[exc].astype(np.int32), tgt[exc].astype(np.int32), synapse_type=0, weight=0.5,
                           delay=delay))
    net.connect(Connection(src[~exc].astype(np.int32), tgt[~exc].astype(np.int32), synapse_type=1, weight=2.5,
                           delay=delay))
    ids = np.arange(n, dtype=np.int32)
    net.connect(Connection(ids + n, ids, synapse_type=0, weight=0.5, delay=1))
    return net, SimulationConfig(steps=steps, timestep=0.1)


IZH_NOISE_PER_MS = 5.0


def izhikevich_stdp(n: int = 100_000, in_degree: int = 100, steps: int = 100_000, seed: int = 1,
                    noise_sigma: float | None = None, dt: float = 0.1) -> tuple[Network, SimulationConfig]:
    """Configuration 1: Izhikevich (RK4, current pulses, noise) with pair STDP.
    ``noise_sigma`` is the per-step current sigma; the default scales the
    per-millisecond sigma of 5 to the step: 5 * sqrt(1 ms / dt)."""
    if noise_sigma is None:
        noise_sigma = IZH_NOISE_PER_MS * float(np.sqrt(1.0 / dt))
    rng = np.random.default_rng(seed)
    n_exc = (n * 4) // 5
    net = Network()
    common = {"c": float32(-65.0), "v0": float32(-65.0), "V_th": float32(30.0), "noise_sigma": float32(noise_sigma)}
    net.add_layer(NeuronLayer("IzhikevichCurrentRK4", n_exc, output=True,
                              parameters={"a": float32(0.02), "b": float32(0.2), "d": float32(8.0), **common}))
    net.add_layer(NeuronLayer("IzhikevichCurrentRK4", n - n_exc, output=True,
                              parameters={"a": float32(0.1), "b": float32(0.2), "d": float32(2.0), **common}))
    net.add_learning_rule(LearningRule("STDP", {"Max_LTP": float32(0.1), "LTP_tau": float32(20.0),
                                                "Max_LTD": float32(0.12), "LTD_tau": float32(20.0)}))
    tgt = np.repeat(np.arange(n, dtype=np.int32), in_degree)
    src = rng.integers(0, n - 1, size=n * in_degree, dtype=np.int64)
    src = (src + (src >= tgt)).astype(np.int32)  # skip self
    delay_ms = rng.integers(1, 21, size=n * in_degree)
    delay = np.rint(delay_ms / dt).astype(np.int32)  # 10..200 steps at dt = 0.1 ms
    exc = src < n_exc
    net.connect(Connection(src[exc], tgt[exc], synapse_type=0, weight=6.0, max_weight=10.0, delay=delay[exc],
                           synapse_rule=0))
    net.connect(Connection(src[~exc], tgt[~exc], synapse_type=1, weight=5.0, delay=delay[~exc]))
    return net, SimulationConfig(steps=steps, timestep=dt)


def batched_sizes(instances: int = 256, lo: int = 500, hi: int = 50_000, seed: int = 3) -> np.ndarray:
    rng = np.random.default_rng(seed)
    return np.rint(np.exp(rng.uniform(np.log(lo), np.log(hi), size=instances))).astype(np.int64)


def lif_instance_arrays(n: int, seed: int, in_degree: float = 100.0) -> tuple[np.ndarray, np.ndarray]:
    """Seeded Erdos-Renyi recurrent connectivity of one batched-LIF instance
    (local ids, no autapses, no multapses) with p = in_degree/(n-1): a dense
    Bernoulli mask for n <= 4096, else Binomial(n(n-1), p) uniform pairs with
    duplicates dropped."""
    rng = np.random.default_rng(seed)
    p = min(1.0, in_degree / max(1, n - 1))
    if n <= 4096:
        mask = rng.random((n, n)) < p
        np.fill_diagonal(mask, False)
        src, tgt = np.nonzero(mask)
        return src.astype(np.int32), tgt.astype(np.int32)
    m = int(rng.binomial(n * (n - 1), p))
    src = rng.integers(0, n, size=m, dtype=np.int64)
    tgt = rng.integers(0, n - 1, size=m, dtype=np.int64)
    tgt = tgt + (tgt >= src)
    key = src * n + tgt
    key.sort()
    key = key[np.concatenate(([True], key[1:] != key[:-1]))]  # drop multapses
    return (key // n).astype(np.int32), (key % n).astype(np.int32)


def _instance_layers(n: int, rate_hz: float) -> list[NeuronLayer]:
    return [_lif_layer(n), NeuronLayer.poisson_rate(n, rate_bias_hz=rate_hz, rate_gain_hz_per_current=0.0)]


def _instance_arrays(n: int, seed: int, offset: int = 0, delay: int = 15):
    """(source, target, type, weight, delay) of one instance, ids from offset:
    recurrent E (+0.5) / I (type 1, 2.5) synapses, then the 1:1 Poisson drive."""
    src, tgt = lif_instance_arrays(n, seed)
    n_exc = (n * 4) // 5
    inh = src >= n_exc
    ids = np.arange(n, dtype=np.int32)
    s = np.concatenate([src, ids + n]) + offset
    t = np.concatenate([tgt, ids]) + offset
    ty = np.concatenate([inh.astype(np.int32), np.zeros(n, np.int32)])
    w = np.concatenate([np.where(inh, 2.5, 0.5).astype(np.float32), np.full(n, 0.5, np.float32)])
    d = np.concatenate([np.full(len(src), delay, np.int32), np.ones(n, np.int32)])
    return s.astype(np.int32), t.astype(np.int32), ty, w, d


def batched_params(instances: int = 256, lo: int = 500, hi: int = 50_000, seed: int = 3):
    """Instance sizes (log-uniform) and Poisson drive rates (uniform 4-12 kHz)."""
    sizes = batched_sizes(instances, lo, hi, seed)
    rates = np.random.default_rng(seed + 1).uniform(4000.0, 12000.0, size=instances)
    return sizes, rates


def batched_instance(k: int, instances: int = 256, lo: int = 500, hi: int = 50_000, seed: int = 3
                     ) -> NetworkDescription:
    """Instance k alone: a LIF layer and its Poisson layer, connectivity seed
    1000 + k.  The PoissonRate hash index stays local to the instance's
    Poisson layer, as in the reference."""
    sizes, rates = batched_params(instances, lo, hi, seed)
    n = int(sizes[k])
    s, t, ty, w, d = _instance_arrays(n, 1000 + k)
    return NetworkDescription.from_arrays(_instance_layers(n, float(rates[k])), s, t, ty, w, delay=d)


def batched_union(instances: int = 256, lo: int = 500, hi: int = 50_000, seed: int = 3) -> NetworkDescription:
    """All instances as one network of disjoint blocks (instance k at an id
    offset), the form the batched engine runs in one launch per block."""
    sizes, rates = batched_params(instances, lo, hi, seed)
    layers, parts = [], []
    offset = 0
    for k, n in enumerate(sizes):
        n = int(n)
        layers += _instance_layers(n, float(rates[k]))
        parts.append(_instance_arrays(n, 1000 + k, offset))
        offset += 2 * n
    cat = [np.concatenate([p[i] for p in parts]) for i in range(5)]
    return NetworkDescription.from_arrays(layers, cat[0], cat[1], cat[2], cat[3], delay=cat[4])


def batched_lif(instances: int = 256, lo: int = 500, hi: int = 50_000, steps: int = 1000, seed: int = 3
                ) -> tuple[list[NetworkDescription], NetworkDescription, SimulationConfig]:
    """Configuration 2 at small scale (tests): (per-instance descriptions, the
    batched union, config)."""
    singles = [batched_instance(k, instances, lo, hi, seed) for k in range(instances)]
    return singles, batched_union(instances, lo, hi, seed), SimulationConfig(steps=steps, timestep=0.1)
