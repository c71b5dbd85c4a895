"""GPU engine vs the CPU oracle on identical seeded inputs (bit-exact).

Every comparison here is exact: spike rasters, membrane traces, final state,
weights and STDP traces, and the delivered-event multiset.  The engine is
built with -fmad=false and the oracle with -ffp-contract=off, and arrivals
are applied per target in the same canonical (CSC) order, so every float
operation matches.  Size-independent properties (determinism, composition of
run calls, invariance to launch shape, instance independence in a batch) are
checked at larger sizes.
"""
import ctypes
import os

import numpy as np
import pytest

import neuronbridge_gb300 as nb
from neuronbridge_gb300 import _lib, workloads

pytestmark = pytest.mark.gpu


def _oracle(net, cfg, **kw):
    import oracle

    return oracle.OracleNet(net.to_native().flat(cfg.timestep, **kw))


def _raster_equal(a, b):
    (ta, ia), (tb, ib) = a, b
    return len(ta) == len(tb) and np.array_equal(ta, tb) and np.array_equal(ia, ib)


def _output_mask(net):
    d = net.to_native()
    return np.repeat(d.layer_output, d.layer_count)


def _oracle_raster(o, net):
    """Oracle spikes of output layers ordered by (time, id): the engine
    records output layers only, as the reference's output spike buffer."""
    t, i = o.spikes()
    keep = _output_mask(net)[i]
    t, i = t[keep], i[keep]
    order = np.lexsort((i, t))
    return t[order], i[order]


def test_plain_lif_10k_steps_bit_exact(oracle_lib):
    net, cfg = workloads.plain_lif()  # 1000 LIF + 1000 Poisson, 10,000 steps
    trace_ids = np.arange(0, 1000, 100)
    sim = nb.Simulation(net, cfg)
    sim.set_trace(trace_ids)
    sim.run()
    o = _oracle(net, cfg)
    o.set_trace(trace_ids)
    o.run(cfg.steps)
    assert sim.next_time == o.next_time == cfg.steps + 1
    assert _raster_equal(sim.spike_raster(), _oracle_raster(o, net))
    assert np.array_equal(sim.traces(), o.traces().astype(np.float32))
    assert np.array_equal(sim.state_field(0), o.state(0).astype(np.float32))
    assert np.array_equal(sim.state_field(6), o.state(6).astype(np.float32))
    assert sim.num_events == o.num_events > 0
    assert sim.block_steps == 15  # Poisson drive is a generator: blocking over the 15-step delay


def test_delivered_event_multiset_bit_exact(oracle_lib):
    net, cfg = workloads.plain_lif(steps=400)
    sim = nb.Simulation(net, cfg, event_log_capacity=2_000_000)
    sim.run(400)
    o = _oracle(net, cfg)
    o.set_event_log(True)
    o.run(400)
    gt, gc, gw = sim.logged_events()
    ot, oc, ow = o.events()
    g = np.lexsort((gc, gt))
    k = np.lexsort((oc, ot))
    assert len(gt) == len(ot) > 0
    assert np.array_equal(gt[g], ot[k]) and np.array_equal(gc[g], oc[k])
    assert np.array_equal(gw[g], ow[k].astype(np.float32))


def test_izhikevich_stdp_small_bit_exact(oracle_lib):
    net, cfg = workloads.izhikevich_stdp(n=3000, in_degree=100)
    sim = nb.Simulation(net, cfg, seed=2)
    sim.set_trace([0, 1, 2999])
    sim.run(3000)
    o = _oracle(net, cfg, seed=2)
    o.set_trace([0, 1, 2999])
    o.run(3000)
    assert _raster_equal(sim.spike_raster(), _oracle_raster(o, net))
    assert len(sim.spike_raster()[0]) > 0
    assert np.array_equal(sim.traces(), o.traces().astype(np.float32))
    for f in (0, 1, 6):
        assert np.array_equal(sim.state_field(f), o.state(f).astype(np.float32)), f
    gw = sim.weights()
    ow, oa, ob, ol = o.weights()
    assert np.array_equal(gw["weight"], ow.astype(np.float32))
    assert np.array_equal(gw["apre"], oa.astype(np.float32))
    assert np.array_equal(gw["apost"], ob.astype(np.float32))
    assert np.array_equal(gw["last_update"], ol)
    assert not np.array_equal(gw["weight"], net.to_native().weight)  # STDP moved weights


def test_izhikevich_full_size_1000_steps_bit_exact(oracle_lib):
    """The headline network itself -- 100k neurons, 10M synapses (8M plastic),
    delays 10..200 steps, noise, pair STDP -- over its first 1,000 steps
    (1,001 updates): several recurrent round trips with STDP acting.  Raster,
    the membrane potential of ten neurons at every step, the final v, u and
    LastSpike of every neuron, and every synapse's weight, Apre, Apost and
    last-update step are bit-identical to the oracle."""
    net, cfg = workloads.izhikevich_stdp()
    trace_ids = np.arange(0, 100_000, 10_000)
    sim = nb.Simulation(net, cfg, seed=2)
    sim.set_trace(trace_ids)
    sim.run(1000)
    o = _oracle(net, cfg, seed=2).set_threads(os.cpu_count() or 1)
    o.set_trace(trace_ids)
    o.run(1000)
    assert sim.next_time == o.next_time == 1001
    g_raster = sim.spike_raster()
    assert len(g_raster[0]) > 50_000  # ~7 spikes per ms of the 100k network
    assert _raster_equal(g_raster, _oracle_raster(o, net))
    assert sim.num_events == o.num_events
    tr = sim.traces()
    assert tr.shape == (1001, 10)
    assert np.array_equal(tr, o.traces().astype(np.float32))
    for f in (0, 1, 6):  # v, u, LastSpike
        assert np.array_equal(sim.state_field(f), o.state(f).astype(np.float32)), f
    gw = sim.weights()
    ow, oa, ob, ol = o.weights()
    assert np.array_equal(gw["weight"], ow.astype(np.float32))
    assert np.array_equal(gw["apre"], oa.astype(np.float32))
    assert np.array_equal(gw["apost"], ob.astype(np.float32))
    assert np.array_equal(gw["last_update"], ol)
    plastic = net.to_native().rule >= 0
    moved = gw["weight"][plastic] != np.float32(6.0)
    assert moved.sum() > 100_000  # STDP acted on many synapses


def _first_divergence(a, b):
    """First step at which two (time, id) rasters hold different spike sets
    (None if they are equal)."""
    (ta, ia), (tb, ib) = a, b
    ka = np.unique(ta.astype(np.int64) << 32 | ia.astype(np.int64))
    kb = np.unique(tb.astype(np.int64) << 32 | ib.astype(np.int64))
    diff = np.setxor1d(ka, kb, assume_unique=True)
    return None if len(diff) == 0 else int(diff.min() >> 32)


# FP32 against the FP64 oracle (the same discretised dynamics, every float
# operation in double): the benchmark spec's membrane tolerance is 1e-5 relative.
MEMBRANE_REL_TOL = 1e-5


@pytest.mark.parametrize("config", ["plain_lif", "izhikevich_stdp"])
def test_fp32_error_against_fp64_oracle(oracle_lib, config):
    """The engine's FP32 run against the FP64 oracle.  The membrane traces of
    ten neurons stay within MEMBRANE_REL_TOL of FP64 at every step up to the
    first step at which the rasters differ.  Plain LIF: the rasters agree over
    at least the first 1,000 steps (2,977 measured) and the spike counts of
    the 10,000 steps are within 0.5 % (119,889 against 120,025 measured).  Izhikevich + STDP at 100k neurons is chaotic (noise,
    recurrent excitation): one threshold crossing among 100k neurons flips
    within the first 100 steps (step 48 measured), after which the spike
    counts still agree within 0.1 % over 1,000 steps."""
    import oracle

    if config == "plain_lif":
        net, cfg = workloads.plain_lif()
        steps, trace_ids, kw = cfg.steps, np.arange(0, 1000, 100), {}
    else:
        net, cfg = workloads.izhikevich_stdp()
        steps, trace_ids, kw = 1000, np.arange(0, 100_000, 10_000), {"seed": 2}
    sim = nb.Simulation(net, cfg, **kw)
    sim.set_trace(trace_ids)
    sim.run(steps)
    o64 = oracle.OracleNet(net.to_native().flat(cfg.timestep, **kw), precision=64).set_threads(os.cpu_count() or 1)
    o64.set_trace(trace_ids)
    o64.run(steps)
    g, r = sim.spike_raster(), _oracle_raster(o64, net)
    fd = _first_divergence(g, r)
    upto = steps + 1 if fd is None else fd  # trace row k is step k
    tr32, tr64 = sim.traces()[:upto].astype(np.float64), o64.traces()[:upto]
    rel = np.abs(tr32 - tr64) / np.maximum(np.abs(tr64), 1e-30)
    assert upto > 10 and rel.max() <= MEMBRANE_REL_TOL, (fd, rel.max())
    n32, n64 = len(g[0]), len(r[0])
    if config == "plain_lif":
        assert fd is None or fd >= 1000, fd
        assert abs(n32 - n64) <= 5e-3 * n64, (n32, n64)
    else:
        assert fd is None or fd >= 10, fd
        assert abs(n32 - n64) <= 1e-3 * n64, (n32, n64)


def test_conductance_izhikevich_kat_on_gpu():
    import json
    import os

    gold = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "numerical_accuracy_kat.json")))
    net = nb.Network().add_layer(nb.NeuronLayer("TimeDrivenIzhikevic_Exponential_Decay", 1, output=True))
    sim = nb.Simulation(net, nb.SimulationConfig(steps=24, timestep=gold["timestep"]))
    sim.set_current_at(1, 0, gold["current"])
    v, u = [], []
    for _ in range(gold["steps"]):
        sim.run(1)
        st = sim.neuron_state(0)["state_variables"]
        v.append(st[0])
        u.append(st[1])
    assert np.array_equal(np.float32(v), np.float32(gold["izhikevich"]["expected_v"]))
    assert np.array_equal(np.float32(u), np.float32(gold["izhikevich"]["expected_u"]))


def test_dense_semantics_profile(oracle_lib):
    net, cfg = workloads.plain_lif(n=300, steps=2000)
    sim = nb.Simulation(net, cfg, semantics="dense")
    sim.run()
    o = _oracle(net, cfg, semantics=1)
    o.run(cfg.steps)
    assert _raster_equal(sim.spike_raster(), _oracle_raster(o, net))
    assert np.array_equal(sim.state_field(0), o.state(0).astype(np.float32))


def test_dense_semantics_izhikevich(oracle_lib):
    """Dense-runtime Izhikevich (decay-then-add, u from the new v, V_th given)
    driven by Poisson sources through excitatory and inhibitory synapses."""
    rng = np.random.default_rng(12)
    n, npoi = 400, 200
    net = nb.Network()
    net.add_layer(nb.NeuronLayer("TimeDrivenIzhikevic_Exponential_Decay", n, output=True,
                                 parameters={"V_th": nb.float32(-50.0)}))
    net.add_layer(nb.NeuronLayer.poisson_rate(npoi, rate_bias_hz=200.0, rate_gain_hz_per_current=0.0))
    src = rng.integers(n, n + npoi, size=8000).astype(np.int32)
    tgt = rng.integers(0, n, size=8000).astype(np.int32)
    typ = (rng.random(8000) < 0.25).astype(np.int32)
    net.connect(nb.Connection(src, tgt, synapse_type=typ, weight=rng.uniform(0.01, 0.06, 8000).astype(np.float32),
                              delay=rng.integers(1, 6, 8000).astype(np.int32)))
    cfg = nb.SimulationConfig(steps=1500, timestep=0.5)
    sim = nb.Simulation(net, cfg, semantics="dense")
    sim.run()
    o = _oracle(net, cfg, semantics=1)
    o.run(cfg.steps)
    assert len(sim.spike_raster()[0]) > 0
    assert _raster_equal(sim.spike_raster(), _oracle_raster(o, net))
    for f in (0, 1, 2, 3):
        assert np.array_equal(sim.state_field(f), o.state(f).astype(np.float32)), f


def test_run_calls_compose():
    net, cfg = workloads.plain_lif(n=400, steps=1000)
    a = nb.Simulation(net, cfg)
    a.run(300).run(200).run(1)
    b = nb.Simulation(net, cfg)
    b.run(501)
    assert a.next_time == b.next_time == 502
    assert _raster_equal(a.spike_raster(), b.spike_raster())
    assert np.array_equal(a.state_field(0), b.state_field(0))


def test_launch_shape_invariance():
    net, cfg = workloads.izhikevich_stdp(n=4000, in_degree=50)
    ref = nb.Simulation(net, cfg, seed=2)
    ref.run(1500)
    for kw in ({"block_steps": 1}, {"block_steps": 3, "threads_per_block": 64}, {"threads_per_block": 32},
               {"use_graph": False}):
        s = nb.Simulation(net, cfg, seed=2, **kw)
        s.run(1500)
        assert _raster_equal(ref.spike_raster(), s.spike_raster()), kw
        assert np.array_equal(ref.weights()["weight"], s.weights()["weight"]), kw


def test_batched_union_equals_independent_instances():
    singles, union, cfg = workloads.batched_lif(instances=6, lo=200, hi=3000, steps=500)
    u = nb.Simulation(union, cfg)
    u.run(500)
    ut, ui = u.spike_raster()
    offset = 0
    for net in singles:
        n = net.neuron_count
        s = nb.Simulation(net, cfg)
        s.run(500)
        sel = (ui >= offset) & (ui < offset + n)
        assert _raster_equal((ut[sel], ui[sel] - offset), s.spike_raster())
        offset += n


def test_reset_restores_initial_state():
    net, cfg = workloads.plain_lif(n=200, steps=300)
    s = nb.Simulation(net, cfg)
    s.run()
    r1 = s.spike_raster()
    s.reset()
    s.run()
    assert _raster_equal(r1, s.spike_raster())


def test_weight_get_set_by_original_index():
    net, cfg = workloads.plain_lif(n=100, steps=10)
    s = nb.Simulation(net, cfg)
    w0 = net.to_native().weight
    assert s.get_connection_weight(5) == w0[5]
    s.set_connection_weight(5, 1.25)
    assert s.get_connection_weight(5) == np.float32(1.25)
    with pytest.raises(nb.NbgError):
        s.set_connection_weight(10**9, 1.0)


def test_weight_snapshot_round_trip(tmp_path, oracle_lib):
    """The reference's weight_roundtrip case (set 0.75, save, set 0.15, load
    gives 0.75), then a learned STDP network: its snapshot loaded into a fresh
    simulation reproduces every weight bit, and the loaded simulation keeps
    running exactly as the oracle does from the same weights."""
    import oracle

    net, cfg = workloads.plain_lif(n=100, steps=10)
    s = nb.Simulation(net, cfg)
    path = tmp_path / "weights.dat"
    s.set_connection_weight(0, 0.75).save_weights(path)
    s.set_connection_weight(0, 0.15).load_weights(path)
    assert s.get_connection_weight(0) == np.float32(0.75)
    assert path.read_text().startswith("NPGR_WEIGHT_SNAPSHOT 1\ntime_step ")

    net, cfg = workloads.izhikevich_stdp(n=1000, in_degree=50)
    a = nb.Simulation(net, cfg, seed=2)
    a.run(1000)
    learned = a.weights()["weight"]
    assert not np.array_equal(learned, net.to_native().weight)
    a.save_weights(path)

    b = nb.Simulation(net, cfg, seed=2)
    b.load_weights(path)
    assert np.array_equal(b.weights()["weight"], learned)
    b.run(200)
    desc = net.to_native()
    desc.weight = learned.copy()
    ref = oracle.OracleNet(desc.flat(cfg.timestep, seed=2))
    ref.run(200)
    assert np.array_equal(b.weights()["weight"], ref.weights()[0].astype(np.float32))
    assert _raster_equal(b.spike_raster(), _oracle_raster(ref, net))

    bad = tmp_path / "short.dat"
    bad.write_text("NPGR_WEIGHT_SNAPSHOT 1\ntime_step 0\nblock main 0 1\nrle\n1 0.5\nend_block\nend\n")
    with pytest.raises(RuntimeError, match="LoadWeight failed: main weight block count does not match"):
        b.load_weights(bad)


def test_nbnet_path_simulation_equals_in_memory(tmp_path, oracle_lib):
    """Simulation(path) streams a .nbnet file (small memory budget, several
    batches) into the same engine state as Simulation(network)."""
    from neuronbridge_gb300 import nbnet

    net, cfg = workloads.izhikevich_stdp(n=3000, in_degree=60)
    path = tmp_path / "izh.nbnet"
    nbnet.from_network(net, path)
    a = nb.Simulation(net, cfg, seed=2)
    b = nb.Simulation(path, cfg, seed=2, build_options=nbnet.StreamingBuildOptions(memory_budget_mb=1))
    assert b.build_stats["runtime_build_path"] == "streaming_direct"
    assert b.build_stats["connection_count"] == 180000
    a.run(800)
    b.run(800)
    assert _raster_equal(a.spike_raster(), b.spike_raster())
    assert np.array_equal(a.weights()["weight"], b.weights()["weight"])
    assert np.array_equal(a.state_field(0), b.state_field(0))


def _decay_table(sim, rules):
    n = ctypes.c_int64()
    _lib.check(sim.lib.nbg_get_decay_table(sim._h, 0, 0, 0, None, ctypes.byref(n)))
    tab = np.zeros((rules, 2, n.value), np.float32)
    for r in range(rules):
        for w in range(2):
            _lib.check(sim.lib.nbg_get_decay_table(sim._h, r, w, n.value,
                                                   tab[r, w].ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                                   ctypes.byref(n)))
    return tab


def test_dense_profile_stdp_uses_device_expf(oracle_lib):
    """Dense-runtime STDP: decay factors from CUDA's expf with
    inv_tau = 1/max(1e-6, tau) (DenseLearningDeviceRuntime.cuh:65-77), built
    on the device; the oracle, given the same factors, is bit-exact.  The
    factors stay within 2 ulp of the host libm table of the legacy profile
    (CUDA documents a 2-ulp bound for expf)."""
    import oracle

    net, cfg = workloads.izhikevich_stdp(n=2000, in_degree=50)
    dense = nb.Simulation(net, cfg, seed=2, semantics="dense")
    legacy = nb.Simulation(net, cfg, seed=2)
    td, tl = _decay_table(dense, 1), _decay_table(legacy, 1)
    n = min(td.shape[-1], tl.shape[-1])
    ulp = np.abs(td[..., :n].view(np.int32).astype(np.int64) - tl[..., :n].view(np.int32).astype(np.int64))
    assert ulp.max() <= 2 and td[..., -1].max() == 0.0
    dense.run(1500)
    o = oracle.OracleNet(net.to_native().flat(cfg.timestep, semantics=1, seed=2))
    o.set_decay_table(td)
    o.run(1500)
    assert _raster_equal(dense.spike_raster(), _oracle_raster(o, net))
    assert np.array_equal(dense.weights()["weight"], o.weights()[0].astype(np.float32))
    assert not np.array_equal(dense.weights()["weight"], net.to_native().weight)


def test_bench_profiling_totals_and_reset():
    net, cfg = workloads.plain_lif(n=200, steps=100)
    sim = nb.Simulation(net, cfg)
    sim.run(300)
    first = sim.bench_profiling_snapshot()["device_ms"]
    sim.run(200)
    p = sim.bench_profiling_snapshot()
    assert p["run_calls"] == 2 and p["simulated_steps"] == 501
    assert abs(p["total_device_ms"] - (first + p["device_ms"])) < 1e-9
    assert p["total_kernel_launches"] >= 2
    sim.reset_bench_profiling()
    z = sim.bench_profiling_snapshot()
    assert z["run_calls"] == 0 and z["total_device_ms"] == 0.0
    assert sim.publish_output() is sim and sim.flush() is sim
