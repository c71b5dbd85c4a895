"""Benchmark: synaptic events/s on one GB300 for the 100k-neuron Izhikevich +
pair-STDP network (RK4, dt = 0.1 ms, 10M synapses).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
                    [--workload izh|lif|batched|dense|adjoint]

The default workload is the headline (izh).  The others measure the remaining
configurations with the same timing rules and print one JSON line each:
lif (1,000 LIF + Poisson), batched (256 LIF instances in one engine vs one
engine per instance), dense (64 x 8192 LIF, split-BF16 tensor-core delivery
vs the FP32 CUDA-core path, error vs FP64), adjoint (recurrent LIF forward +
hand-written adjoint, B=128, T=1000).

One benchmark step = one run call of 10,000 simulation steps (1 s of
simulated time) through the public API; the default K = 10 covers the
configuration's 10 s.  Warm-up steps advance the same simulation first.

`value` is delivered synaptic events per second of device time (CUDA events on
the engine's stream, summed over the K timed run calls; inputs resident in HBM).
`e2e` is the same count divided by the host wall time of the K
`Simulation.run()` calls, which include every per-call host<->device copy (the
control words up, the spike raster down).  The L2 cache is flushed (a 256 MiB
write) between timed iterations.

With --impl reference the CPU oracle port (oracle/, a restatement of the
reference's CPU path; the reference itself does not build here) is timed on a
bounded sample of the same workload on the host cores.

N > 1 (torchrun): the headline network does not shard, so every rank runs an
independent replica; `value` sums the events of all ranks over the slowest
rank's time.  The batched workload shards its instances over the ranks
(greedy size-balanced bin packing, neuronbridge_gb300/partition.py) and
reports strong scaling; lif, dense and adjoint run on rank 0 alone.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

SIM_STEPS_PER_BENCH_STEP = 10_000
# algorithmic bytes (per unit) for the update kernel and the delivery path:
#   neuron-step: v,u read+write 16 B, ring word read+clear 8 B, spike/refractory 8 B
#   delivered event: plastic 40 B (index 4, weight r/w 8, Apre/Apost/last r/w 24,
#   mask bit 4), non-plastic 12 B; post-STDP: 36 B per (post spike x plastic in-synapse)
BYTES_PER_NEURON_STEP = 32
BYTES_PER_LIF_NEURON_STEP = 24  # V r/w 8, refractory counter r/w 8, ring word read+clear 8
BYTES_PER_PLASTIC_EVENT = 40
BYTES_PER_STATIC_EVENT = 12
BYTES_PER_POST_UPDATE = 36
# DRAM bytes (read + write) of one k_update launch of this workload (10 steps x
# 100k neurons) from an ncu capture of that launch with a cold L2
# (30.24 MB read + 0.16 MB written)
KUPDATE_TRAFFIC_BYTES = 30.39e6
# DRAM bytes (read + write) of one k_update launch of the 256-instance batched
# workload (15 steps), scaled from an ncu capture on its first 32 instances
BATCHED_TRAFFIC_BYTES = 2.478e9  # 267.7 MB on 282,235 LIF neurons x 2,612,540 / 282,235 (256 x 15 launches)
# DRAM bytes (read + write) of one dense step launch (64 x 8192, delivery and
# update) from an ncu capture with a cold L2
DENSE_TRAFFIC_BYTES = 277.5e6
# device -> host bytes of a run call besides its raster entries (8 B each: step
# and id) and traces: error word, raster cursor, ordered-entry count (4 B each)
# and the delivered-event counter read by num_events (8 B)
RUN_CALL_D2H_BYTES = 4 + 4 + 4 + 8


def _peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        d = json.load(open(path))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    def __init__(self, index: int = 0):
        self.index = index
        self.rows: list[list[str]] = []
        self.proc = None

    def start(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self) -> dict:
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        rows = [r for r in self.rows if len(r) >= 7]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[0]) for r in rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[3 + k].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def _dist():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def _host_cpu() -> str:
    """Host CPU model (lscpu / /proc/cpuinfo) for the CPU-side numbers."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for key in ("Model name:", "BIOS Model name:"):
            for line in out.splitlines():
                if line.strip().startswith(key):
                    return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return "unknown"


def _post_fanout(desc) -> np.ndarray:
    """plastic in-degree per neuron"""
    return np.bincount(desc.target[desc.rule >= 0], minlength=desc.neuron_count)


def headline_config(sim_steps: int, world: int) -> dict:
    """`config` of the headline workload, shared by both arms (the GPU engine
    and the CPU reference arm) so that they describe the same work.  The
    launch shape the GPU arm tunes is reported beside it, not in it."""
    from neuronbridge_gb300 import workloads

    return {"workload": "izhikevich_stdp_100k", "neurons": 100_000, "synapses": 10_000_000,
            "plastic_synapses": 7_999_283, "sim_steps_per_step": sim_steps, "dt_ms": 0.1, "integrator": "rk4",
            "noise_sigma_per_step": round(workloads.IZH_NOISE_PER_MS * float(np.sqrt(1.0 / 0.1)), 4),
            "noise": "N(0, 5^2) per ms as a per-step Irwin-Hall(12) draw, sigma 5*sqrt(1 ms/dt) = 15.81 per "
                     "0.1-ms step (sigma 5 per step leaves the network silent; see sigma5_per_step)",
            "connectivity_rng": "numpy PCG64 seed 1 (not mt19937_64); in-degree 100, sources drawn with "
                                "replacement (about 5% multapses), self excluded",
            "l2": "flushed between timed iterations (256 MiB write)",
            "parallelism": "replicas" if world > 1 else "single"}


def cpu_baseline_sample(sim_steps: int = 3000) -> dict:
    """The oracle port on the same 100k/10M network for a bounded number of
    simulation steps, OpenMP over all host cores (identical results to one
    thread: each thread owns disjoint neurons and synapses)."""
    import oracle
    from neuronbridge_gb300 import workloads

    cores = os.cpu_count() or 1
    net, cfg = workloads.izhikevich_stdp()
    o = oracle.OracleNet(net.to_native().flat(cfg.timestep, seed=2)).set_threads(cores)
    t0 = time.perf_counter()
    o.run(sim_steps)
    dt = time.perf_counter() - t0
    return {"value": o.num_events / dt, "unit": "synaptic events/s", "cores": cores, "kind": "port",
            "sample": f"100k-neuron Izhikevich+STDP network, first {sim_steps + 1} simulation steps, "
                      f"oracle FP32 restatement, OpenMP over {cores} host threads",
            "neuron_steps_per_s": 100_000 * (sim_steps + 1) / dt, "seconds": dt}


def sigma5_sample(args, local: int, choice: dict | None) -> dict:
    """The headline network with the literal per-step noise sigma of 5 (the
    same connectivity, seeds and launch shape): the network stays silent, so
    a step is the neuron update and the empty drain alone.  Three run calls of
    args.sim_steps after one warm-up call, CUDA events on the engine stream."""
    import neuronbridge_gb300 as nb
    from neuronbridge_gb300 import workloads

    net, cfg = workloads.izhikevich_stdp(noise_sigma=5.0)
    sim = nb.Simulation(net, cfg, device=local, seed=2)
    if choice:
        sim.set_launch(int(choice["threads_per_block"]), int(choice["block_steps"]))
    sim.run(args.sim_steps)
    sim.clear_spikes()
    dev = 0.0
    launches = ev = spikes = 0
    calls = 3
    for _ in range(calls):
        e0 = sim.num_events
        sim.run(args.sim_steps)
        p = sim.bench_profiling_snapshot()
        dev += p["device_ms"] / 1e3
        launches += p["kernel_launches"]
        ev += sim.num_events - e0
        spikes += len(sim.spike_raster()[0])
        sim.clear_spikes()
    sim.close()
    n = 100_000
    return {"noise_sigma_per_step": 5.0, "neuron_steps_per_s": n * args.sim_steps * calls / dev,
            "synaptic_events_per_s": ev / dev, "spikes": int(spikes), "sim_steps": args.sim_steps * calls,
            "avg_launch_us": 1e6 * dev / max(1, launches), "launches": int(launches)}


def phase_split(neuron_bytes: float, delivery_bytes: float, dev_s: float, launches: int, silent: dict,
                peak: float) -> dict:
    """Roofline fractions of the two phases of k_update.  The neuron update
    (with the drain of an empty arrival ring) is timed on the silent sigma-5
    network, the same launches with no spike and no arrival; delivery + STDP
    is the rest of the headline launch.  Each phase's algorithmic bytes over
    its time, against the measured HBM peak."""
    t_launch = dev_s / max(1, launches)
    t_upd = silent["avg_launch_us"] * 1e-6
    t_del = t_launch - t_upd
    upd = neuron_bytes / max(1, launches) / t_upd / 1e9
    out = {"method": "update = launch time of the same network at noise sigma 5 per step (silent); "
                     "delivery + STDP = headline launch time minus that",
           "update": {"launch_us": 1e6 * t_upd, "achieved": upd, "frac": upd / peak,
                      "bytes_per_launch": neuron_bytes / max(1, launches)}}
    if t_del > 0:
        dl = delivery_bytes / max(1, launches) / t_del / 1e9
        out["delivery_stdp"] = {"launch_us": 1e6 * t_del, "achieved": dl, "frac": dl / peak,
                                "bytes_per_launch": delivery_bytes / max(1, launches)}
    return out


def fp64_error_sample(local: int, steps: int = 1000) -> dict:
    """FP32 error against the FP64 oracle on the headline network: the
    engine's first `steps` steps (a fresh simulation, membrane potential of
    ten neurons every step) against the oracle's FP64 build of the same
    discretised dynamics.  The oracle is the checker here, not the measured
    path.  The network is chaotic, so the rasters part at some step; the
    membrane error is taken over the steps before it."""
    import oracle
    import neuronbridge_gb300 as nb
    from neuronbridge_gb300 import workloads

    net, cfg = workloads.izhikevich_stdp()
    trace_ids = np.arange(0, 100_000, 10_000)
    sim = nb.Simulation(net, cfg, device=local, seed=2)
    sim.set_trace(trace_ids)
    sim.run(steps)
    t32, i32 = sim.spike_raster()
    tr32 = sim.traces().astype(np.float64)
    sim.close()
    o = oracle.OracleNet(net.to_native().flat(cfg.timestep, seed=2), precision=64).set_threads(os.cpu_count() or 1)
    o.set_trace(trace_ids)
    o.run(steps)
    t64, i64 = o.spikes()
    tr64 = o.traces()
    k32 = np.unique(t32.astype(np.int64) << 32 | i32.astype(np.int64))
    k64 = np.unique(t64.astype(np.int64) << 32 | i64.astype(np.int64))
    diff = np.setxor1d(k32, k64, assume_unique=True)
    fd = None if len(diff) == 0 else int(diff.min() >> 32)
    upto = tr32.shape[0] if fd is None else fd
    err = np.abs(tr32[:upto] - tr64[:upto])
    rel = err / np.maximum(np.abs(tr64[:upto]), 1e-30)
    return {"updates": int(tr32.shape[0]), "traced_neurons": len(trace_ids),
            "first_raster_divergence_step": fd, "steps_compared": int(upto),
            "membrane_max_abs_mV": float(err.max()), "membrane_median_abs_mV": float(np.median(err)),
            "membrane_max_rel": float(rel.max()), "spikes_fp32": int(len(k32)), "spikes_fp64": int(len(k64)),
            "spike_pairs_differing": int(len(diff))}


def run_reference(args) -> None:
    world, rank, _ = _dist()
    if rank != 0:
        return
    per_step = []
    events = 0
    import oracle
    from neuronbridge_gb300 import workloads

    cores = os.cpu_count() or 1
    net, cfg = workloads.izhikevich_stdp()
    o = oracle.OracleNet(net.to_native().flat(cfg.timestep, seed=2)).set_threads(cores)
    # the same windows as the GPU arm: W warm-up run calls then K timed ones,
    # each args.sim_steps simulation steps, from the same initial state; a
    # 256 MiB host write between timed windows, as the GPU arm flushes its L2
    sample = args.sim_steps
    flush = np.empty(256 * 1024 * 1024 // 8, np.float64)
    for k in range(args.warmup + args.steps):
        e0 = o.num_events
        t0 = time.perf_counter()
        o.run(sample)
        dt = time.perf_counter() - t0
        if k >= args.warmup:
            per_step.append(dt)
            events += o.num_events - e0
            flush.fill(1.0)
    total = sum(per_step)
    value = events / total
    line = {
        "impl": "reference", "metric": "synaptic events/s", "value": value, "unit": "synaptic events/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": headline_config(sample, world),
        "cpu_baseline": {"value": value, "unit": "synaptic events/s", "cores": cores, "kind": "port",
                         "host_cpu": _host_cpu(),
                         "sample": f"the GPU arm's windows: {args.warmup} warm-up and {args.steps} timed run calls "
                                   f"of {sample} simulation steps of the 100k/10M network, oracle FP32 restatement "
                                   "(the reference's CPU path does not build here: it needs Boost and its CMake "
                                   f"build), OpenMP over {cores} host threads"},
        "e2e": {"value": value, "unit": "synaptic events/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def _launch_shape(sim, args, trial_steps: int) -> dict:
    """The update kernel's launch shape: autotuned, or fixed by --launch
    THREADSxSTEPS (profiling runs, where the tuning launches would come first)."""
    from neuronbridge_gb300 import tuning

    if args.launch:
        threads, steps = (int(x) for x in args.launch.lower().split("x"))
        sim.set_launch(threads, steps)
        return {"choice": {"threads_per_block": threads, "block_steps": sim.block_steps, "ms": None, "fixed": True}}
    return tuning.autotune(sim, trial_steps=trial_steps)


def _common(args, metric, value, unit, ms_per_step, config, **extra):
    line = {"metric": metric, "value": value, "unit": unit, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": config}
    line.update(extra)
    return line


def bench_lif(args) -> dict:
    """1,000 LIF + 1,000 Poisson: one benchmark step = one run(10,000) call."""
    import torch

    import neuronbridge_gb300 as nb
    from neuronbridge_gb300 import tuning, workloads

    net, cfg = workloads.plain_lif()
    # no per-launch events: they would sit between the launches of the graph
    # and stretch it; the only kernel of the call is k_update, so the call's
    # device time over its launches is the launch duration
    sim = nb.Simulation(net, cfg)
    tune = _launch_shape(sim, args, 1000)  # launch shape only; resets the simulation
    trace_ids = np.arange(0, 1000, 100)  # V of neurons 0, 100, ..., 900 every step, with the raster
    sim.set_trace(trace_ids)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    for _ in range(args.warmup):
        sim.run(cfg.steps)
        sim.clear_spikes()
        flush.fill_(1.0)
    ev = dev = upd = wall = 0.0
    launches = spikes = 0
    clocks = ClockSampler(0)
    clocks.start()
    for _ in range(args.steps):
        e0 = sim.num_events
        w0 = time.perf_counter()
        sim.run(cfg.steps)
        wall += time.perf_counter() - w0
        spikes += len(sim.spike_raster()[0])
        p = sim.bench_profiling_snapshot()
        ev += sim.num_events - e0
        dev += p["device_ms"] / 1e3
        upd += p["device_ms"] / 1e3
        launches += p["kernel_launches"] + p["raster_order_launches"]
        sim.clear_spikes()
        flush.fill_(1.0)
    clk = clocks.stop()
    n = 2000
    upd_bytes = 24 * 1000 * cfg.steps * args.steps + 12 * ev
    peak, kind = _peaks()
    return _common(args, "synaptic events/s", ev / dev, "synaptic events/s", 1e3 * dev / args.steps,
                   {"workload": "plain_lif_1k", "neurons": n, "sim_steps_per_step": cfg.steps,
                    "block_steps": sim.block_steps, "tuned": tune["choice"],
                    "recorded": "raster of the LIF layer and V of neurons 0, 100, ..., 900 every step"},
                   neuron_steps_per_s=n * cfg.steps * args.steps / dev,
                   roofline={"bound": "hbm", "kernel": "k_update", "achieved": upd_bytes / upd / 1e9, "peak": peak,
                             "unit": "GB/s", "frac": upd_bytes / upd / 1e9 / peak, "peak_kind": kind,
                             "traffic": None},
                   e2e={"value": ev / wall, "unit": "synaptic events/s", "h2d_bytes_per_step": 16,
                        "d2h_bytes_per_step": int(8 * spikes / args.steps + 4 * len(trace_ids) * cfg.steps
                                                 + RUN_CALL_D2H_BYTES)},
                   gpu_launches=int(launches), clocks=clk)


def bench_batched(args) -> dict | None:
    """256 LIF instances (500..50,000 neurons each): one engine over the
    union, autotuned launch shape, one graph per run(1,000) call, against the
    same 256 networks each in its own engine, run one after the other.

    Under torchrun the instances shard over the ranks by greedy size-balanced
    bin packing (every rank builds one batched engine over its share; no
    data-path collective): the total work is fixed, so the scaling is strong.
    `value` sums the events of all ranks over the slowest rank's device time."""
    import torch

    import neuronbridge_gb300 as nb
    from neuronbridge_gb300 import workloads
    from neuronbridge_gb300.partition import partition_instances, shard_loads
    from neuronbridge_gb300.replicas import aggregate

    world, rank, local = _dist()
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    sizes, _ = workloads.batched_params(args.instances)
    shards = partition_instances(sizes, world)
    mine = shards[rank]
    t0 = time.perf_counter()
    singles = [workloads.batched_instance(int(k), args.instances) for k in mine]
    build_s = time.perf_counter() - t0
    cfg = nb.SimulationConfig(steps=1000, timestep=0.1)
    n_lif = int(sizes[mine].sum())
    ev = dev = wall = 0.0
    launches = 0
    raster = {"order_ms": 0.0, "download_ms": 0.0, "append_ms": 0.0, "order_launches": 0}
    raster_entries = 0
    tune = {"choice": None}
    block_steps = None
    clk = None
    if len(mine):
        sim = nb.Simulation.batch(singles, cfg, device=local)  # one engine over the shard (nbg_create_batch)
        tune = _launch_shape(sim, args, 300)
        for _ in range(args.warmup):
            sim.run(cfg.steps)
            sim.clear_spikes()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    if len(mine):
        clocks = ClockSampler(local)
        clocks.start()
        for _ in range(args.steps):
            e0 = sim.num_events
            w0 = time.perf_counter()
            sim.run(cfg.steps)
            wall += time.perf_counter() - w0
            p = sim.bench_profiling_snapshot()
            ev += sim.num_events - e0
            dev += p["device_ms"] / 1e3
            launches += p["kernel_launches"]
            for k in raster:
                raster[k] += p["raster_" + k]
            raster_entries += sim._num_raster()  # downloaded as (step, id) int32 pairs
            sim.clear_spikes()
        clk = clocks.stop()
        block_steps = sim.block_steps
        del sim
    torch.cuda.synchronize()
    # plain form: every instance in its own engine, one after another
    p_ev = p_dev = p_wall = 0.0
    for net in singles:
        s = nb.Simulation(net, cfg, device=local)
        s.run(cfg.steps)  # warm (first call: steps + 1 updates)
        e0 = s.num_events
        w0 = time.perf_counter()
        s.run(cfg.steps)
        p_wall += time.perf_counter() - w0
        p_ev += s.num_events - e0
        p_dev += s.bench_profiling_snapshot()["device_ms"] / 1e3
        s.close()
    # the Poisson layers have no inputs: the engine evaluates them inline at
    # their targets, so the neuron-steps are the LIF neurons'
    upd_bytes = BYTES_PER_LIF_NEURON_STEP * n_lif * cfg.steps * args.steps + BYTES_PER_STATIC_EVENT * ev
    dev_dev = f"cuda:{local}" if world > 1 else None
    (dev_all, wall_all, p_dev_all, p_wall_all), (ev_all, p_ev_all, bytes_all) = aggregate(
        [dev, wall, p_dev, p_wall], [ev, p_ev, upd_bytes], device=dev_dev)
    if rank != 0:
        return None
    value = ev_all / dev_all
    plain = p_ev_all / p_dev_all
    peak, kind = _peaks()
    per_launch = launches / args.steps
    # per GPU: every rank's algorithmic bytes over the slowest rank's device
    # time, divided by the ranks (the same totals and clock as `value`)
    achieved = bytes_all / dev_all / world / 1e9
    loads = shard_loads(sizes, shards)
    config = {"workload": f"batched_lif_{args.instances}", "instances": args.instances,
              "lif_neurons": int(sizes.sum()), "sim_steps_per_step": cfg.steps, "block_steps": block_steps,
              "tuned": tune["choice"], "host_build_s": build_s,
              "l2": "inputs larger than L2 (2.2 GB of synapse columns per launch)",
              "parallelism": "single" if world == 1 else
              f"instances sharded over {world} ranks (greedy size-balanced bin packing)"}
    if world > 1:
        config["shard_instances"] = [int(len(s)) for s in shards]
        config["shard_lif_neurons"] = [int(x) for x in loads]
    line = _common(args, "synaptic events/s", value, "synaptic events/s", 1e3 * dev_all / args.steps, config,
                   neuron_steps_per_s=int(sizes.sum()) * cfg.steps * args.steps / dev_all,
                   roofline={"bound": "hbm", "kernel": "k_update<Spec<1, 0>> (LIF, static; Poisson generators "
                                                       "packed eight per thread)",
                             "achieved": achieved, "peak": peak, "unit": "GB/s",
                             "frac": achieved / peak, "peak_kind": kind,
                             "scope": "per GPU" if world == 1 else
                             f"per GPU: all {world} ranks' bytes / slowest rank's time / {world}",
                             "traffic": (BATCHED_TRAFFIC_BYTES if args.instances == 256 and world == 1 else None),
                             "traffic_unit": "bytes per launch (ncu on 32 instances, scaled by units)",
                             "algorithmic_bytes_per_launch": upd_bytes / (per_launch * args.steps),
                             "avg_update_launch_us": 1e6 * dev / launches if launches else None},
                   plain={"value": plain, "unit": "synaptic events/s", "device_s_per_1000_steps": p_dev_all,
                          "wall_s_per_1000_steps": p_wall_all},
                   speedup_vs_plain=value / plain,
                   e2e={"value": ev_all / wall_all, "unit": "synaptic events/s", "h2d_bytes_per_step": 16,
                        "d2h_bytes_per_step": int(8 * raster_entries / max(1, args.steps) + RUN_CALL_D2H_BYTES)},
                   raster_per_run_call={k: v / max(1, args.steps) for k, v in raster.items()},
                   gpu_launches=int(launches + raster["order_launches"]), clocks=clk)
    line["n_gpus"] = world
    if world > 1:
        line["scaling"] = "strong"
    return line


def bench_dense(args) -> dict:
    """64 instances x 8,192 LIF sharing W (N(0, 1/8192)); one benchmark step =
    run(500).  Split-BF16 tensor-core delivery vs the FP32 CUDA-core path, and
    the delivery error of both against FP64 S W on the spike matrices of the
    run (sampled every benchmark step)."""
    import torch

    from neuronbridge_gb300 import NeuronLayer
    from neuronbridge_gb300.dense import DensePopulations, dense_weights
    from neuronbridge_gb300.workloads import LIF_PARAMS

    n, per = 8192, (args.per or 500)
    w = dense_weights(n)
    layer = NeuronLayer("TimeDrivenLIF_Voltage_jump", 1, parameters=dict(LIF_PARAMS))
    w64 = torch.from_numpy(w).double().cuda()
    out = {}
    for prec in ("split_bf16", "split_bf16_sync", "fp32"):
        eng = DensePopulations(w, layer, precision=prec)
        for _ in range(args.warmup):
            eng.run(per)
        dev = dl = 0.0
        errs = []
        clocks = ClockSampler(0)
        clocks.start()
        for _ in range(args.steps):
            eng.run(per)
            p = eng.profile()
            dev += p["device_ms"] / 1e3
            dl += p["delivery_ms"] / 1e3
            s = eng.spikes()
            got = eng.deliver(s)
            ref = (torch.from_numpy(s).double().cuda() @ w64).cpu().numpy()
            errs.append(float(np.abs(got - ref).max()))
        clk = clocks.stop()
        out[prec] = {"ms_per_step": 1e3 * dev / (args.steps * per), "delivery_us": 1e6 * dl / (args.steps * per),
                     "max_abs_err_vs_fp64": max(errs), "clocks": clk,
                     "spikes_per_step": float(eng.spike_counts()[-per:].mean())}
        del eng
    sp = out["split_bf16"]
    byts = 2 * 2 * n * n + 64 * n * 2 + 2 * 64 * n * 4
    flops = 2 * 64 * n * n * 2
    peak, kind = _peaks()
    achieved = byts / (sp["delivery_us"] * 1e-6) / 1e9
    return _common(args, "steps/s", 1e3 / sp["ms_per_step"], "steps/s", sp["ms_per_step"] * per,
                   {"workload": "dense_split_bf16_64x8192", "instances": 64, "neurons": n, "sim_steps_per_step": per},
                   neuron_steps_per_s=64 * n * 1e3 / sp["ms_per_step"],
                   roofline={"bound": "hbm", "kernel": "k_dense_umma<LifFinish> (split-BF16 delivery + LIF, tcgen05)",
                             "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                             "peak_kind": kind, "traffic": DENSE_TRAFFIC_BYTES if n == 8192 else None,
                             "traffic_unit": "bytes per launch (ncu, cold L2, one step)",
                             "algorithmic_bytes_per_launch": byts,
                             "tflops": flops / (sp["delivery_us"] * 1e-6) / 1e12},
                   paths=out)


def bench_adjoint(args) -> dict:
    """Recurrent LIF (256 -> 1024 -> 10, B = 128, T = 1000): forward alone,
    and forward + hand-written adjoint backward, per training step."""
    import torch

    from neuronbridge_gb300.adjoint import RECORD_BUDGET_BYTES, RecurrentLIF, poisson_inputs, record_bytes

    model = RecurrentLIF()  # records every step's state (1.7 GB): no replay in the backward
    rates = torch.empty(256).uniform_(5.0, 50.0, generator=torch.Generator().manual_seed(5))
    x = poisson_inputs(rates, 1000, 128, dt=1.0, seed=5)
    labels = torch.randint(0, 10, (128,), generator=torch.Generator().manual_seed(6)).cuda()
    lossf = torch.nn.functional.cross_entropy

    def fwd():
        with torch.no_grad():
            return lossf(model(x), labels)

    def step():
        model.zero_grad(set_to_none=True)
        loss = lossf(model(x), labels)
        loss.backward()
        return loss

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        fwd()
    e1.record()
    torch.cuda.synchronize()
    f_ms = e0.elapsed_time(e1) / args.steps
    e0.record()
    for _ in range(args.steps):
        step()
    e1.record()
    torch.cuda.synchronize()
    t_ms = e0.elapsed_time(e1) / args.steps
    gflop = 2 * 128 * (256 * 1024 + 1024 * 1024 + 1024 * 10) * 1000 / 1e9
    return _common(args, "training steps/s", 1e3 / t_ms, "steps/s", t_ms,
                   {"workload": "adjoint_rlif_b128_t1000", "batch": 128, "T": 1000, "n_rec": 1024,
                    "segment": 100, "record": record_bytes(1000, 128, 1024) <= RECORD_BUDGET_BYTES},
                   forward_ms=f_ms, backward_ms=t_ms - f_ms, backward_over_forward=(t_ms - f_ms) / f_ms,
                   forward_tflops=gflop / f_ms)


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--sim-steps", type=int, default=SIM_STEPS_PER_BENCH_STEP)
    ap.add_argument("--workload", default="izh", choices=["izh", "lif", "batched", "dense", "adjoint"])
    ap.add_argument("--instances", type=int, default=256, help="batched workload: number of instances")
    ap.add_argument("--launch", default=None, help="fixed update-kernel launch shape THREADSxSTEPS (no autotune)")
    ap.add_argument("--per", type=int, default=None, help="simulation steps per benchmark step (dense)")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    if args.impl == "reference":
        run_reference(args)
        return
    if args.workload != "izh":
        if args.workload == "batched":
            line = bench_batched(args)
            if line is not None:
                print(json.dumps(line), flush=True)
            return
        if _dist()[1] != 0:
            return  # lif, dense and adjoint measure one GPU: rank 0 alone runs them
        fn = {"lif": bench_lif, "dense": bench_dense, "adjoint": bench_adjoint}
        print(json.dumps(fn[args.workload](args)), flush=True)
        return

    world, rank, local = _dist()
    import torch

    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)

    import neuronbridge_gb300 as nb
    from neuronbridge_gb300 import tuning, workloads

    net, cfg = workloads.izhikevich_stdp()
    desc = net.to_native()
    # no per-launch events (they would sit between the graph's launches and
    # stretch it): k_update is the only kernel of a run call, so the call's
    # device time (CUDA events on the engine stream) over its launch count is
    # the average launch duration
    sim = nb.Simulation(desc, cfg, device=local, seed=2)
    tune = _launch_shape(sim, args, 500)  # launch shape only; resets the simulation
    fan = _post_fanout(desc)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")

    def bench_step():
        e0 = sim.num_events
        t0 = time.perf_counter()
        sim.run(args.sim_steps)
        wall = time.perf_counter() - t0
        prof = sim.bench_profiling_snapshot()
        ev = sim.num_events - e0
        _, ids = sim.spike_raster()
        sim.clear_spikes()
        return ev, wall, prof, ids, len(ids)

    raster = {"order_ms": 0.0, "download_ms": 0.0, "append_ms": 0.0, "order_launches": 0}

    for _ in range(args.warmup):
        bench_step()
        flush.fill_(1.0)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clocks = ClockSampler(local)
    clocks.start()
    tot_ev = tot_wall = tot_dev = tot_upd = 0.0
    tot_spk = tot_post = 0
    launches = 0
    for _ in range(args.steps):
        ev, wall, prof, new_ids, nspk = bench_step()
        tot_ev += ev
        tot_wall += wall
        tot_dev += prof["device_ms"] / 1e3
        tot_upd += prof["device_ms"] / 1e3
        tot_spk += nspk
        tot_post += int(fan[new_ids].sum())
        launches += prof["kernel_launches"]
        for k in raster:
            raster[k] += prof["raster_" + k]
        flush.fill_(1.0)
    torch.cuda.synchronize()
    clk = clocks.stop()
    from neuronbridge_gb300.replicas import aggregate

    (tot_dev, tot_wall), (tot_ev_all,) = aggregate([tot_dev, tot_wall], [tot_ev], device=f"cuda:{local}")
    if rank != 0:
        return

    n = desc.neuron_count
    sim_steps = args.steps * args.sim_steps
    plastic_frac = float(np.mean(desc.rule >= 0))
    neuron_bytes = BYTES_PER_NEURON_STEP * n * sim_steps
    delivery_bytes = (tot_ev * (plastic_frac * BYTES_PER_PLASTIC_EVENT + (1 - plastic_frac) * BYTES_PER_STATIC_EVENT)
                      + BYTES_PER_POST_UPDATE * tot_post)
    upd_bytes = neuron_bytes + delivery_bytes
    peak, peak_kind = _peaks()
    achieved = upd_bytes / tot_upd / 1e9 if tot_upd > 0 else None
    silent = sigma5_sample(args, local, tune["choice"])
    value = tot_ev_all / tot_dev
    d2h = 8 * (tot_spk / args.steps) + RUN_CALL_D2H_BYTES
    line = {
        "metric": "synaptic events/s", "value": value, "unit": "synaptic events/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot_dev / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded network, in-kernel noise)",
        "config": headline_config(args.sim_steps, world),
        "launch_shape": {"block_steps": sim.block_steps, "tuned": tune["choice"]},
        "neuron_steps_per_s": n * sim_steps * world / tot_dev,
        "spikes_per_s_simulated": tot_spk / (sim_steps * 1e-4) / n,
        "roofline": {"bound": "hbm", "kernel": "k_update (drain + RK4 + STDP + spike propagation)",
                     "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": (achieved / peak) if achieved else None, "peak_kind": peak_kind,
                     "traffic": KUPDATE_TRAFFIC_BYTES if args.sim_steps % 10 == 0 else None,
                     "traffic_unit": "bytes per launch (ncu, cold L2)",
                     "algorithmic_bytes_per_launch": upd_bytes / max(1, launches),
                     "avg_update_launch_us": 1e6 * tot_upd / max(1, launches)},
        "phases": phase_split(neuron_bytes, delivery_bytes, tot_upd, launches, silent, peak),
        "sigma5_per_step": silent,
        "e2e": {"value": tot_ev_all / tot_wall, "unit": "synaptic events/s", "h2d_bytes_per_step": 4 + 8 + 4,
                "d2h_bytes_per_step": int(d2h)},
        "raster_per_run_call": {k: v / args.steps for k, v in raster.items()},
        "gpu_launches": int(launches + raster["order_launches"]),
        "clocks": clk,
    }
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline_sample()
        line["fp64_error"] = fp64_error_sample(local)
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
