"""Launch-shape autotuner for the step engine.

Results never depend on the launch shape (the parity tests run the same
network at several shapes and compare bit for bit); only speed does.  The
tuner times each candidate (threads per block x steps per update launch) on
the live network with CUDA events (``bench_profiling_snapshot``), keeps the
fastest, and resets the simulation to its initial state afterwards.
"""
from __future__ import annotations

from .simulation import Simulation


def candidates(block_limit: int) -> list[tuple[int, int]]:
    steps = sorted({block_limit, max(1, block_limit // 2), max(1, (2 * block_limit) // 3)}, reverse=True)
    # 32-thread blocks let the block scheduler spread a small network's warps
    # evenly over the SMs (one wave, no SM holding a whole extra block)
    return [(t, b) for t in (128, 256, 64, 32) for b in steps]


def autotune(sim: Simulation, trial_steps: int = 300, repeats: int = 2) -> dict:
    """Pick the fastest (threads_per_block, block_steps) for `sim` and reset it.
    Each candidate is run once to build its graph, then timed `repeats` times
    over `trial_steps` simulation steps; the score is the best device time."""
    limit = sim.block_steps
    results = []
    for threads, b in candidates(limit):
        sim.set_launch(threads, b)
        sim.run(trial_steps)
        best = float("inf")
        for _ in range(repeats):
            sim.run(trial_steps)
            best = min(best, sim.bench_profiling_snapshot()["device_ms"])
        results.append({"threads_per_block": threads, "block_steps": b, "ms": best})
    pick = min(results, key=lambda r: r["ms"])
    sim.reset()
    sim.set_launch(pick["threads_per_block"], pick["block_steps"])
    return {"choice": pick, "trials": results, "trial_steps": trial_steps}
