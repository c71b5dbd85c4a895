"""Simulation.batch (nbg_create_batch): independent networks in one engine
give, per instance, exactly what each gives alone -- spikes, state, learned
weights and events -- and the engine places them as the host union does."""
import numpy as np
import pytest

import neuronbridge_gb300 as nb
from neuronbridge_gb300 import workloads

from test_batch_cpu import _plastic_net

pytestmark = pytest.mark.gpu


def _parts():
    singles, _, _ = workloads.batched_lif(instances=5, lo=150, hi=1500, steps=400)
    return singles + [_plastic_net(300, 7, 20.0), _plastic_net(120, 8, 40.0)]


def test_batch_equals_instances_alone():
    parts = _parts()
    cfg = nb.SimulationConfig(steps=400, timestep=0.1)
    batch = nb.Simulation.batch(parts, cfg)
    assert batch.instance_count == len(parts)
    batch.run()
    events = 0
    for k, p in enumerate(parts):
        alone = nb.Simulation(p, cfg)
        alone.run()
        ta, ia = alone.spike_raster()
        tb, ib = batch.instance_raster(k)
        assert np.array_equal(ta, tb) and np.array_equal(ia, ib), k
        for f in (0, 4, 6):
            assert np.array_equal(alone.state_field(f), batch.instance_state(k, f)), (k, f)
        assert np.array_equal(alone.weights()["weight"], batch.instance_weights(k)), k
        events += alone.num_events
        alone.close()
    assert batch.num_events == events
    assert len(batch.spike_raster()[0]) > 0

