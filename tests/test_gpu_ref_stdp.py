"""The engine's pair STDP against the reference's own STDP code.

The golden cases of tests/golden/stdp_reference.json (produced by the
reference's STDP.cpp / STDP_State.cpp, see tests/test_oracle_ref_stdp.py)
run on the GPU as networks of input-spike neurons (tests/stdp_pin_cases.py):
the weight after every event tick and the final Apre, Apost and LastUpdate
equal the reference's bit for bit."""
import numpy as np
import pytest

import neuronbridge_gb300 as nb
import stdp_pin_cases as pin

pytestmark = pytest.mark.gpu

CASES = pin.load_cases()


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_engine_matches_reference_stdp(case):
    net, times, ids = pin.network(case)
    sim = nb.Simulation(net, nb.SimulationConfig(steps=case["ticks"], timestep=case["dt"]))
    sim.add_external_spikes(times, ids)
    n = len(case["w0"])
    want = dict(zip(case["event_ticks"], np.asarray(case["w_at_event_ticks"], np.float32)))
    checked = 0
    sim.run(1)  # updates t = 0, 1
    t = 1
    while True:
        if t in want:
            w = sim.weights()["weight"][:n]
            assert np.array_equal(w, want[t]), (t, w, want[t])
            checked += 1
        if t == case["ticks"] - 1:
            break
        # run to the next event tick in one call
        nxt = min([x for x in want if x > t] + [case["ticks"] - 1])
        sim.run(nxt - t)
        t = nxt
    assert checked == len(want)
    st, si = sim.spike_raster()
    assert st[si == n + 1].tolist() == case["post"]
    g = sim.weights()
    assert np.array_equal(g["apre"][:n], np.float32(case["apre"]))
    assert np.array_equal(g["apost"][:n], np.float32(case["apost"]))
    assert np.array_equal(g["last_update"][:n], np.int32(case["last_update"]))
