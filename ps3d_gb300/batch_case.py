"""Batched workload: many independent runs of uneven grid sizes.

    python -m ps3d_gb300.batch_case --steps 500

96 runs by default (48 x 32^3, 32 x 64^3, 16 x 128^3), each the Beltrami
flow plus its own seeded perturbation with an amplitude drawn log-uniformly
in [1e-4, 1e-2] and prediss drawn from {10, 30, 60, 90}, mixed form,
impl-diff-rk4.  Every run's step is one captured CUDA graph; the runs'
graphs are interleaved on their own streams (ps3d_gpu_batch_advance).  For
comparison, `--compare K` also times K host-driven steps of every run, one
run after another.  Prints one JSON line: grid points x steps per second of
the whole batch.
"""
import argparse
import json
import sys
import time

import numpy as np

from . import Ps3dGpu, batch_advance, ic


def build(counts, seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    runs = []
    k = 0
    for n, cnt in counts:
        for _ in range(cnt):
            amp = float(10.0 ** rng.uniform(-4.0, -2.0))
            pre = float(rng.choice([10.0, 30.0, 60.0, 90.0]))
            vor, pert = ic.beltrami_plus_perturbation(n, n, n, seed=1000 + k, amplitude=amp)
            m = Ps3dGpu(n, n, n, ic.BELTRAMI_BOX["lower"], ic.BELTRAMI_BOX["extent"], precision="mixed",
                        prediss=pre, cflmax=0.5, nnu=3, pretype="vorch")
            m.setup_fields(vor, pert)
            runs.append((n, amp, pre, m))
            k += 1
    return runs


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--steps", type=int, default=500)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--compare", type=int, default=10)
    ap.add_argument("--counts", default="32:48,64:32,128:16")
    ap.add_argument("--seed", type=int, default=7)
    a = ap.parse_args(argv)
    counts = [tuple(int(x) for x in c.split(":")) for c in a.counts.split(",")]
    t0 = time.perf_counter()
    runs = build(counts, a.seed)
    setup_s = time.perf_counter() - t0
    models = [r[3] for r in runs]
    pts = sum(n ** 3 for n, _, _, _ in runs)
    ts = [0.0] * len(models)
    ts, _ = batch_advance(models, ts, a.warmup)
    ts, ms = batch_advance(models, ts, a.steps)
    value = pts * a.steps / (ms * 1e-3) / 1e6
    comp = None
    if a.compare > 0:
        # the same runs advanced by host-driven steps, one run after another
        for m in models:
            m.synchronize()
        t1 = time.perf_counter()
        for i, m in enumerate(models):
            for _ in range(a.compare):
                ts[i], _ = m.advance(ts[i])
        sec = time.perf_counter() - t1
        comp = {"steps": a.compare, "value": pts * a.compare / sec / 1e6,
                "how": "ps3d_gpu_advance per run, runs one after another, wall clock"}
    diag = [m.energy_series() for m in models[:3]]
    print(json.dumps({
        "metric": "Mpts*steps/s", "value": value, "unit": "Mpts*steps/s", "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": ms / a.steps, "runs": len(models), "points_per_step": pts,
        "config": {"workload": "batched Beltrami+perturbation runs, mixed, impl-diff-rk4",
                   "counts": {f"{n}^3": c for n, c in counts}},
        "host_driven_sequential": comp, "setup_s": setup_s,
        "sample_energy_series": diag,
    }), flush=True)
    for m in models:
        m.close()


if __name__ == "__main__":
    sys.exit(main())
