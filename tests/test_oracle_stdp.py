"""Pair STDP in the oracle against a direct pure-Python restatement of
STDP.cpp:19-61 / STDP_State.cpp:17-26 on a small pre/post schedule (the
scenario of the reference's pair_stdp_gpu_trajectory.cpp: one plastic
synapse, weight 8, max 20, dt 1 ms; pre spikes at ticks 0 and 7)."""
import ctypes
import ctypes.util

import numpy as np

_libm = ctypes.CDLL(ctypes.util.find_library("m"))
_libm.expf.restype = ctypes.c_float
_libm.expf.argtypes = [ctypes.c_float]


def _expf(x):
    """std::exp(float) as the reference calls it (STDP_State.cpp:21-23)."""
    return np.float32(_libm.expf(float(x)))

from neuronbridge_gb300 import Connection, LearningRule, Network, NeuronLayer, float32


def _py_stdp(events, w0, wmax, a_plus, tau_p, a_minus, tau_m, dt):
    f = np.float32
    # STDP_State.cpp:5-7: 1.0 / (float member) evaluated in double, stored as float
    inv_p, inv_m = f(1.0 / float(f(tau_p))), f(1.0 / float(f(tau_m)))
    apre = apost = f(0.0)
    last = 0
    w = f(w0)
    out = []
    for t, kind in events:
        dtime = f(f(t - last) * f(dt))
        apre = f(apre * _expf(f(-dtime * inv_p)))
        apost = f(apost * _expf(f(-dtime * inv_m)))
        last = t
        if kind == "pre":
            apre = f(apre + f(1.0))
            w = f(w + f(-f(a_minus) * apost))
        else:
            apost = f(apost + f(1.0))
            w = f(w + f(f(a_plus) * apre))
        w = f(0.0) if w < 0 else (f(wmax) if w > wmax else w)
        out.append(float(w))
    return out


def test_single_synapse_trajectory(oracle_lib):
    import oracle

    # neuron 0: Poisson source firing at p=1 only while driven; simpler: a
    # PoissonRate that always fires (rate 1e6) pre-synaptic, and a target LIF
    # that fires every update (V_th below rest) -> dense pre/post schedule.
    net = Network()
    net.add_layer(NeuronLayer("PoissonRate", 1, parameters={"rate_bias_hz": float32(1e6)}))
    net.add_layer(NeuronLayer("TimeDrivenLIF_Voltage_jump", 1,
                              parameters={"V_th": float32(-100.0), "t_ref": 0, "V_reset": float32(-5.0)}))
    net.add_learning_rule(LearningRule("STDP", {"Max_LTP": float32(0.92), "LTP_tau": float32(16.8),
                                                "Max_LTD": float32(0.53), "LTD_tau": float32(33.1)}))
    net.connect(Connection(0, 1, synapse_type=0, weight=8.0, max_weight=20.0, delay=3, synapse_rule=0))
    sim = oracle.OracleNet(net.to_native().flat(1.0))
    sim.run(12)  # updates t = 0..12
    w, apre, apost, last = sim.weights()
    # expected event order: post at every t (target fires each update), pre
    # arrivals at t = 3..12 (source fires every t, delay 3); pre before post.
    events = []
    for t in range(13):
        if t >= 3:
            events.append((t, "pre"))
        events.append((t, "post"))
    exp = _py_stdp(events, 8.0, 20.0, 0.92, 16.8, 0.53, 33.1, 1.0)
    assert np.float32(w[0]) == np.float32(exp[-1])
    assert last[0] == 12
