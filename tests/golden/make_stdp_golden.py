"""Golden pair-STDP trajectories produced by the reference's own STDP code.

The reference's STDP.cpp, STDP_State.cpp and the classes they use are
compiled from the reference tree by oracle/ref_stdp/Makefile (oracle/_ref,
test infrastructure; needs a copy of the reference on this machine, the
Makefile's REF or NBG_REFERENCE_ROOT).  Each case below replays a seeded
pre/post event schedule on one post-synaptic neuron through that code and
records the weights after every tick that holds an event, and the final
Apre, Apost and LastUpdate of every connection.

    python tests/golden/make_stdp_golden.py

Output: tests/golden/stdp_reference.json (committed), read by
tests/test_oracle_ref_stdp.py to pin the oracle's STDP without the reference.
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def cases() -> list[dict]:
    """Event schedules.  A pre event of connection k at tick t is the arrival
    of a spike sent at t - delay[k]; post ticks are at least two apart and at
    least 1 (a forced spike of the target, see the test)."""
    out = []
    # the reference fixture's setting (pair_stdp_gpu_trajectory.cpp:31-52):
    # one connection, weight 8, max 20, dt 1 ms, the STDP defaults
    # (STDP.h:14-20); pre arrivals at ticks 1 and 8 (its interface spikes at
    # ticks 0 and 7 over a delay-1 synapse), post spikes around them
    pre = np.zeros((16, 1), np.uint8)
    pre[[1, 8], 0] = 1
    post = np.zeros(16, np.uint8)
    post[[2, 9, 12]] = 1
    out.append({"name": "fixture_single", "dt": 1.0, "params": [0.92, 16.8, 0.53, 33.1], "w0": [8.0],
                "wmax": [20.0], "delay": [1], "pre": pre, "post": post})
    rng = np.random.default_rng(11)
    # the headline network's rule (A+ 0.1, A- 0.12, tau 20 ms, clip [0, 10],
    # weight 6, dt 0.1 ms): six connections, delays 10..200 steps, sparse
    # random trains over 3,000 ticks (gaps of hundreds of steps)
    ticks, n = 3000, 6
    delay = rng.integers(10, 201, size=n)
    pre = (rng.random((ticks, n)) < 0.004).astype(np.uint8)
    for k in range(n):
        pre[: delay[k], k] = 0
    post = _post_train(rng, ticks, 0.004)
    out.append({"name": "headline_rule", "dt": 0.1, "params": [0.1, 20.0, 0.12, 20.0], "w0": [6.0] * n,
                "wmax": [10.0] * n, "delay": delay.tolist(), "pre": pre, "post": post})
    # strong rule and dense trains: both clamps (0 and w_max) are reached
    ticks, n = 400, 4
    delay = rng.integers(1, 6, size=n)
    pre = (rng.random((ticks, n)) < 0.08).astype(np.uint8)
    for k in range(n):
        pre[: delay[k], k] = 0
    post = _post_train(rng, ticks, 0.08)
    out.append({"name": "clamped", "dt": 1.0, "params": [3.0, 5.0, 4.0, 12.0], "w0": [2.0, 5.0, 9.0, 0.5],
                "wmax": [10.0, 10.0, 12.0, 3.0], "delay": delay.tolist(), "pre": pre, "post": post})
    return out


def _post_train(rng, ticks: int, p: float) -> np.ndarray:
    post = np.zeros(ticks, np.uint8)
    t = 1
    while t < ticks:
        if rng.random() < p:
            post[t] = 1
            t += 2
        else:
            t += 1
    return post


def main() -> None:
    import oracle

    if oracle.build_ref() is None:
        sys.exit("the reference tree is not on this machine (set NBG_REFERENCE_ROOT)")
    res = []
    for c in cases():
        traj, apre, apost, last = oracle.ref_stdp_run(c["w0"], c["wmax"], *c["params"], c["dt"], c["pre"], c["post"])
        ev = np.nonzero(c["pre"].any(axis=1) | c["post"].astype(bool))[0]
        res.append({"name": c["name"], "dt": c["dt"], "params": c["params"], "w0": c["w0"], "wmax": c["wmax"],
                    "delay": c["delay"], "ticks": int(len(c["post"])),
                    "pre": [np.nonzero(c["pre"][:, k])[0].tolist() for k in range(c["pre"].shape[1])],
                    "post": np.nonzero(c["post"])[0].tolist(),
                    "event_ticks": ev.tolist(), "w_at_event_ticks": traj[ev].astype(float).tolist(),
                    "apre": apre.astype(float).tolist(), "apost": apost.astype(float).tolist(),
                    "last_update": last.tolist()})
    dst = os.path.join(HERE, "stdp_reference.json")
    with open(dst, "w") as f:
        json.dump({"source": "reference STDP.cpp / STDP_State.cpp compiled by oracle/ref_stdp/Makefile",
                   "cases": res}, f)
    print("wrote", dst)


if __name__ == "__main__":
    main()
