"""The oracle's pair STDP pinned to the reference's own STDP code.

tests/golden/stdp_reference.json holds weight trajectories and final trace
states that the reference's STDP.cpp / STDP_State.cpp produced (compiled from
the reference tree by oracle/ref_stdp/Makefile, replayed by
tests/golden/make_stdp_golden.py): one case modelled on the reference's
pair_stdp_gpu_trajectory.cpp fixture, the headline network's rule on six
connections over 3,000 ticks, and a strong rule that reaches both clamps.
The oracle runs each schedule as a network (tests/stdp_pin_cases.py) and
must match every weight after every event tick, and the final Apre, Apost
and LastUpdate, bit for bit.  Where the reference tree is on the machine the
reference build is also rerun and must reproduce the fixture."""
import numpy as np
import pytest

import stdp_pin_cases as pin

CASES = pin.load_cases()


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_oracle_matches_reference_stdp(oracle_lib, case):
    import oracle

    net, times, ids = pin.network(case)
    o = oracle.OracleNet(net.to_native().flat(case["dt"]))
    o.add_external_spikes(times, ids)
    n = len(case["w0"])
    want = dict(zip(case["event_ticks"], np.asarray(case["w_at_event_ticks"], np.float32)))
    checked = 0
    o.run(1)  # updates t = 0, 1
    t = 1
    while True:
        if t in want:
            w = o.weights()[0][:n].astype(np.float32)
            assert np.array_equal(w, want[t]), (t, w, want[t])
            checked += 1
        if t == case["ticks"] - 1:
            break
        o.run(1)
        t += 1
    assert checked == len(want)
    # every post event was a spike of the target
    st, si = o.spikes()
    assert st[si == n + 1].tolist() == case["post"]
    w, apre, apost, last = o.weights()
    assert np.array_equal(apre[:n].astype(np.float32), np.float32(case["apre"]))
    assert np.array_equal(apost[:n].astype(np.float32), np.float32(case["apost"]))
    assert np.array_equal(last[:n], np.int32(case["last_update"]))


def test_reference_build_reproduces_fixture():
    import oracle

    if oracle.build_ref() is None:
        pytest.skip("reference tree not on this machine: the committed fixture is the pin")
    import importlib.util
    import os

    spec = importlib.util.spec_from_file_location("make_stdp_golden", os.path.join(os.path.dirname(pin.GOLDEN),
                                                                                 "make_stdp_golden.py"))
    gen = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(gen)
    for c, g in zip(gen.cases(), CASES):
        traj, apre, apost, last = oracle.ref_stdp_run(c["w0"], c["wmax"], *c["params"], c["dt"], c["pre"], c["post"])
        assert np.array_equal(traj[g["event_ticks"]], np.float32(g["w_at_event_ticks"])), c["name"]
        assert np.array_equal(apre, np.float32(g["apre"])) and np.array_equal(apost, np.float32(g["apost"]))
        assert np.array_equal(last, np.int32(g["last_update"]))
