"""Benchmark: synaptic events/s on one GB300 for the 100k-neuron Izhikevich +
pair-STDP network (RK4, dt = 0.1 ms, 10M synapses).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

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

N > 1 (torchrun): the network does not shard, so every rank runs an
independent replica; `value` sums the events of all ranks over the slowest
rank's time.
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
BYTES_PER_PLASTIC_EVENT = 40
BYTES_PER_STATIC_EVENT = 12
BYTES_PER_POST_UPDATE = 36


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


def _post_fanout(desc) -> np.ndarray:
    """plastic in-degree per neuron"""
    return np.bincount(desc.target[desc.rule >= 0], minlength=desc.neuron_count)


def cpu_baseline_sample(sim_steps: int = 1500) -> dict:
    """The oracle port on the same 100k/10M network for a bounded number of
    simulation steps (single host thread)."""
    import oracle
    from neuronbridge_gb300 import workloads

    net, cfg = workloads.izhikevich_stdp()
    o = oracle.OracleNet(net.to_native().flat(cfg.timestep, seed=2))
    t0 = time.perf_counter()
    o.run(sim_steps)
    dt = time.perf_counter() - t0
    return {"value": o.num_events / dt, "unit": "synaptic events/s", "cores": 1, "kind": "port",
            "sample": f"100k-neuron Izhikevich+STDP network, first {sim_steps + 1} simulation steps, "
                      f"oracle FP32 restatement, 1 host thread",
            "neuron_steps_per_s": 100_000 * (sim_steps + 1) / dt, "seconds": dt}


def run_reference(args) -> None:
    world, rank, _ = _dist()
    if rank != 0:
        return
    per_step = []
    events = 0
    import oracle
    from neuronbridge_gb300 import workloads

    net, cfg = workloads.izhikevich_stdp()
    o = oracle.OracleNet(net.to_native().flat(cfg.timestep, seed=2))
    sample = 300  # simulation steps per benchmark step: a bounded sample
    for k in range(args.warmup + args.steps):
        e0 = o.num_events
        t0 = time.perf_counter()
        o.run(sample)
        dt = time.perf_counter() - t0
        if k >= args.warmup:
            per_step.append(dt)
            events += o.num_events - e0
    total = sum(per_step)
    value = events / total
    line = {
        "impl": "reference", "metric": "synaptic events/s", "value": value, "unit": "synaptic events/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "izhikevich_stdp_100k", "neurons": 100_000, "synapses": 10_000_000,
                   "sim_steps_per_step": sample, "dt_ms": 0.1},
        "cpu_baseline": {"value": value, "unit": "synaptic events/s", "cores": 1, "kind": "port",
                         "sample": f"{sample} simulation steps per benchmark step of the 100k/10M network, "
                                   "oracle FP32 restatement (the reference's CPU path does not build here: "
                                   "it needs Boost and its CMake build), 1 host thread"},
        "e2e": {"value": value, "unit": "synaptic events/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--sim-steps", type=int, default=SIM_STEPS_PER_BENCH_STEP)
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    if args.impl == "reference":
        run_reference(args)
        return

    world, rank, local = _dist()
    import torch

    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)

    import neuronbridge_gb300 as nb
    from neuronbridge_gb300 import workloads

    net, cfg = workloads.izhikevich_stdp()
    desc = net.to_native()
    sim = nb.Simulation(desc, cfg, device=local, seed=2, kernel_timing=True)
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

    for _ in range(args.warmup):
        bench_step()
        flush.fill_(1.0)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clocks = ClockSampler(local)
    clocks.start()
    tot_ev = tot_wall = tot_dev = tot_upd = tot_prop = 0.0
    tot_spk = tot_post = 0
    launches = 0
    for _ in range(args.steps):
        ev, wall, prof, new_ids, nspk = bench_step()
        tot_ev += ev
        tot_wall += wall
        tot_dev += prof["device_ms"] / 1e3
        tot_upd += prof["update_kernel_ms"] / 1e3
        tot_prop += prof["propagate_kernel_ms"] / 1e3
        tot_spk += nspk
        tot_post += int(fan[new_ids].sum())
        launches += prof["kernel_launches"]
        flush.fill_(1.0)
    torch.cuda.synchronize()
    clk = clocks.stop()
    if world > 1:
        import torch.distributed as dist

        t = torch.tensor([tot_dev, tot_wall], dtype=torch.float64, device=f"cuda:{local}")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e = torch.tensor([tot_ev], dtype=torch.float64, device=f"cuda:{local}")
        dist.all_reduce(e, op=dist.ReduceOp.SUM)
        tot_dev, tot_wall = float(t[0]), float(t[1])
        tot_ev_all = float(e[0])
    else:
        tot_ev_all = tot_ev
    if rank != 0:
        return

    n = desc.neuron_count
    sim_steps = args.steps * args.sim_steps
    plastic_frac = float(np.mean(desc.rule >= 0))
    upd_bytes = (BYTES_PER_NEURON_STEP * n * sim_steps
                 + tot_ev * (plastic_frac * BYTES_PER_PLASTIC_EVENT + (1 - plastic_frac) * BYTES_PER_STATIC_EVENT)
                 + BYTES_PER_POST_UPDATE * tot_post)
    peak, peak_kind = _peaks()
    achieved = upd_bytes / tot_upd / 1e9 if tot_upd > 0 else None
    value = tot_ev_all / tot_dev
    d2h = 4 * (tot_spk / args.steps) + 4 * (args.sim_steps) + 8 + 8 + 4
    line = {
        "metric": "synaptic events/s", "value": value, "unit": "synaptic events/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot_dev / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded network, in-kernel noise)",
        "config": {"workload": "izhikevich_stdp_100k", "neurons": n, "synapses": int(len(desc.source)),
                   "plastic_synapses": int(np.sum(desc.rule >= 0)), "sim_steps_per_step": args.sim_steps,
                   "dt_ms": 0.1, "integrator": "rk4", "block_steps": sim.block_steps,
                   "l2": "flushed between timed iterations (256 MiB write)", "parallelism": "replicas" if world > 1
                   else "single"},
        "neuron_steps_per_s": n * sim_steps * world / tot_dev,
        "spikes_per_s_simulated": tot_spk / (sim_steps * 1e-4) / n,
        "roofline": {"bound": "hbm", "kernel": "k_update (drain + RK4 + STDP)",
                     "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": (achieved / peak) if achieved else None, "peak_kind": peak_kind,
                     "traffic": None, "update_ms_share": tot_upd / tot_dev if tot_dev else None,
                     "propagate_ms_share": tot_prop / tot_dev if tot_dev else None,
                     "avg_update_launch_us": 1e6 * tot_upd / max(1, launches // 2)},
        "e2e": {"value": tot_ev_all / tot_wall, "unit": "synaptic events/s", "h2d_bytes_per_step": 4 + 8 + 4,
                "d2h_bytes_per_step": int(d2h)},
        "gpu_launches": int(launches),
        "clocks": clk,
    }
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline_sample()
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
