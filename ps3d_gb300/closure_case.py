"""Learned sub-grid closure workload: data, training, evaluation and cost.

    python -m ps3d_gb300.closure_case [--fine 256] [--coarse 64] ...

1. Data.  Fine runs (Beltrami plus a seeded perturbation, prediss 30,
   nnu 3, vorch, Kolmogorov, Hou & Li, CFL 0.5) advance with captured steps;
   every `--sample-every` steps the exact sub-grid tendency
   cut(T_f(omega_f)) - T_c(cut(omega_f)) and the coarse vorticity and velocity
   become one training sample (closure.subgrid_sample).
2. Training: `--iters` Adam steps of the BF16 tensor-core network on the
   device (ps3d_closure_train).
3. Evaluation on held-out seeds: the fine run is the truth; its state cut to
   the coarse grid at t = 0 starts the coarse runs: the plain method
   (hyperdiffusion at prediss 30, the fallback), the closure with the
   hyperdiffusion it replaces set to each --closure-prediss value (0: the
   network is the only sub-grid model), and the same prediss without the
   network.  Kinetic-energy shell spectra (genspec.f90:42-123) of the cut fine
   state and of the coarse runs are compared at the fine run's sample times
   (the coarse spectra interpolated linearly in time between the bracketing
   steps), shells 1..21.  The closure's correction is also compared with the
   exact sub-grid tendency at those states (a-priori error).
4. Cost: device time per unit of model time of the fine run (mixed and,
   with --fp64-cost, FP64) and of the coarse closure run, all with captured
   steps.

Prints one JSON line.
"""
import argparse
import json
import os
import sys
import time

import numpy as np

from . import Ps3dGpu, ic
from .closure import Closure, attach, shell_error, spectral_cut, subgrid_sample

DEFAULT_VARIANTS = ("plain=30,net30_every=30:net+every,net10_every=10:net+every,net30_held=30:net,"
                    "net30_clip=30:net+clip+walls,net0_every=0:net+every,nomodel0=0")

PHYS = dict(prediss=30.0, nnu=3, pretype="vorch", length_scale="Kolmogorov", filtering="Hou & Li", cflmax=0.5)


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def model(n, precision, **kw):
    args = dict(PHYS)
    args.update(kw)
    return Ps3dGpu(n, n, n, ic.BELTRAMI_BOX["lower"], ic.BELTRAMI_BOX["extent"], precision=precision, **args)


def fine_run(n, seed, amplitude, precision):
    m = model(n, precision)
    vor, pert = ic.beltrami_plus_perturbation(n, n, n, seed=seed, amplitude=amplitude)
    m.setup_fields(vor, pert)
    return m


def filtered_spectrum(fine, probe):
    probe.set("svor", spectral_cut(fine.get("svor"), probe.nx, probe.ny, probe.nz))
    probe.vor2vel()
    return probe.ke_spectrum()[0]


def coarse_spectra(m, t_end):
    """Host-driven advances to t_end, (t, spectrum) after every step."""
    t = 0.0
    m.vor2vel()
    out = [(0.0, m.ke_spectrum()[0])]
    while t < t_end:
        t, _ = m.advance(t)
        m.vor2vel()
        out.append((t, m.ke_spectrum()[0]))
    return out


def at_time(series, t):
    ts = np.array([s[0] for s in series])
    i = int(np.searchsorted(ts, t))
    if i == 0:
        return series[0][1]
    if i >= len(ts):
        return series[-1][1]
    t0, t1 = ts[i - 1], ts[i]
    w = (t - t0) / (t1 - t0) if t1 > t0 else 0.0
    a, b = series[i - 1][1], series[i][1]
    k = min(len(a), len(b))
    return (1 - w) * a[:k] + w * b[:k]


def parse_variants(spec):
    """'name=prediss[:opt+opt...],...' -> [(name, prediss, {opts})]"""
    out = []
    for item in spec.split(","):
        name, rest = item.split("=")
        pd, _, opts = rest.partition(":")
        out.append((name.strip(), float(pd), set(o for o in opts.split("+") if o)))
    return out


def cost_per_time(m, t0, nsteps):
    """(device ms per step, mean dt) of nsteps captured steps"""
    t1, _, ms = m.advance_graph(t0, nsteps)
    return ms / nsteps, (t1 - t0) / nsteps


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--fine", type=int, default=256)
    ap.add_argument("--coarse", type=int, default=64)
    ap.add_argument("--train-seeds", type=int, default=8)
    ap.add_argument("--test-seeds", type=int, default=2)
    ap.add_argument("--steps", type=int, default=600)
    ap.add_argument("--sample-every", type=int, default=40)
    ap.add_argument("--amplitude", type=float, default=1.0e-2)
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--iters", type=int, default=3000)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--lr-final", type=float, default=5e-5)
    ap.add_argument("--variants", default=DEFAULT_VARIANTS,
                    help="coarse runs: name=prediss[:option+option...], options net, every, clip, walls, "
                         "g<gain> (the correction times gain), mma (warp-level inference engine instead of "
                         "tcgen05); the first variant with net is timed")
    ap.add_argument("--fp64-cost", action="store_true")
    ap.add_argument("--params-out", default="", help="save the trained network (.npz: params, ct)")
    ap.add_argument("--params-in", default="", help="load a trained network instead of generating data")
    ap.add_argument("--truth-cache", default="",
                    help=".npz of the held-out runs' cut initial states and filtered spectra: read when it "
                         "exists (no fine runs), written otherwise")
    a = ap.parse_args(argv)
    nf, nc = a.fine, a.coarse
    nsamp = 0 if a.params_in else a.train_seeds * (a.steps // a.sample_every + 1)

    coarse = model(nc, "mixed", prediss=0.0)
    net = Closure(nc, nc, nc, max_samples=nsamp, seed=7)
    t_start = time.time()

    # ---------------------------------------------------------------- data
    for s in range(0 if a.params_in else a.train_seeds):
        f = fine_run(nf, 100 + s, a.amplitude, a.precision)
        t = 0.0
        for k in range(0, a.steps + 1, a.sample_every):
            vor, vel, tgt = subgrid_sample(f, coarse)
            net.add_sample(vor, vel, tgt)
            if k + a.sample_every <= a.steps:
                if a.precision == "mixed":
                    t, _, _ = f.advance_graph(t, a.sample_every)
                else:
                    t, _ = f.advance_n(t, a.sample_every)
        log(f"[closure] seed {100 + s}: {net.num_samples} samples, t = {t:.3f}")
        f.close()
    t_data = time.time() - t_start

    # ------------------------------------------------------------ training
    t0 = time.time()
    if a.params_in:
        z = np.load(a.params_in)
        net.set_params(z["params"])
        net.scale = float(z["ct"])
        loss = np.array([np.nan])
        a.iters = 0
    else:
        loss = net.train(a.iters, a.lr, a.lr_final, seed=1)
    t_train = time.time() - t0
    log(f"[closure] trained {a.iters} steps in {t_train:.1f} s: loss {loss[:20].mean():.4f} -> {loss[-50:].mean():.4f}")
    if a.params_out:
        np.savez(a.params_out, params=net.get_params(), ct=net.scale)

    # ---------------------------------------------------------- evaluation
    # coarse variants: the plain method (hyperdiffusion at prediss 30), the
    # closure with the hyperdiffusion it replaces scaled to each
    # --closure-prediss value, and the same without the network
    probe = model(nc, "mixed")
    ct0 = net.scale
    engine0 = net.engine
    variants = parse_variants(a.variants)
    evals = []
    cache = {}
    if a.truth_cache and os.path.exists(a.truth_cache):
        z = np.load(a.truth_cache)
        cache = {k: z[k] for k in z.files}
    for s in range(a.test_seeds):
        key = f"s{900 + s}_"
        if key + "svor0" in cache:
            svor0c, ini = cache[key + "svor0"], cache[key + "ini"]
            times, truth = list(cache[key + "times"]), list(cache[key + "truth"])
            corr = list(cache[key + "corr"])
        else:
            f = fine_run(nf, 900 + s, a.amplitude, a.precision)
            svor0c = spectral_cut(f.get("svor"), nc, nc, nc)
            ini = f.ini_vor_mean
            truth, times, corr = [], [], []
            t = 0.0
            for k in range(0, a.steps + 1, a.sample_every):
                truth.append(filtered_spectrum(f, probe))
                times.append(t)
                vor, vel, tgt = subgrid_sample(f, probe)
                pred = net.predict(vor, vel)
                corr.append(float(np.linalg.norm(pred - tgt) / max(np.linalg.norm(tgt), 1e-300)))
                if k + a.sample_every <= a.steps:
                    if a.precision == "mixed":
                        t, _, _ = f.advance_graph(t, a.sample_every)
                    else:
                        t, _ = f.advance_n(t, a.sample_every)
            f.close()
            kmin = min(len(x) for x in truth)
            cache.update({key + "svor0": svor0c, key + "ini": ini, key + "times": np.array(times),
                          key + "truth": np.array([x[:kmin] for x in truth]), key + "corr": np.array(corr)})
            if a.truth_cache:
                np.savez(a.truth_cache, **cache)
        res = {"seed": 900 + s, "times": [float(x) for x in times], "correction_rel_l2": [float(x) for x in corr],
               "variants": {}, "final_spectra": {"truth": np.asarray(truth[-1])[:22].tolist()}}
        for name, pd, opts in variants:
            use_net = "net" in opts
            m = model(nc, "mixed", prediss=pd)
            m.set("svor", svor0c)
            m.ini_vor_mean = ini
            m.vor2vel()
            te, en, _ = m.energy_series()
            m.init_diffusion(te, en)
            gain = [float(o[1:]) for o in opts if o.startswith("g")]
            if use_net:
                net.scale = ct0 * (gain[0] if gain else 1.0)
                net.engine = "mma" if "mma" in opts else engine0
                attach(m, net, "every" in opts, "clip" in opts, "walls" in opts)
            try:
                sp = coarse_spectra(m, times[-1])
            except Exception as e:  # a variant that blows up is reported, not fatal
                res["variants"][name] = {"failed": str(e)}
                log(f"[closure] test seed {900 + s} {name}: failed ({e})")
                if use_net:
                    attach(m, None)
                m.close()
                continue
            if use_net:
                attach(m, None)
            m.close()
            errs = [shell_error(at_time(sp, tj), et) for tj, et in zip(times, truth)]
            res["variants"][name] = {"max_shell_error": [e[0] for e in errs],
                                     "mean_shell_error": [e[1] for e in errs], "steps": len(sp) - 1}
            res["final_spectra"][name] = at_time(sp, times[-1])[:22].tolist()
            log(f"[closure] test seed {900 + s} {name}: final max / mean shell error "
                f"{errs[-1][0]:.4f} / {errs[-1][1]:.4f} in {len(sp) - 1} steps")
        evals.append(res)
    net.scale = ct0
    net.engine = engine0

    # ---------------------------------------------------------------- cost
    f = fine_run(nf, 900, a.amplitude, "mixed")
    svor0c, ini = spectral_cut(f.get("svor"), nc, nc, nc), f.ini_vor_mean
    ms_f, dt_f = cost_per_time(f, 0.0, 20)
    f.close()
    cost = {"fine_mixed_ms_per_step": ms_f, "fine_dt": dt_f}
    if a.fp64_cost:
        f = fine_run(nf, 900, a.amplitude, "fp64")
        t, ms64 = f.time_advance(0.0, 5)
        cost["fine_fp64_ms_per_step"] = ms64 / 5
        cost["fine_fp64_dt"] = t / 5
        f.close()
    timed = [v for v in variants if "net" in v[2]][:1]
    for name, pd, opts in [("coarse_plain", 30.0, set())] + [("coarse_closure", v[1], v[2]) for v in timed]:
        use_net = "net" in opts
        m = model(nc, "mixed", prediss=pd)
        m.set("svor", svor0c)
        m.ini_vor_mean = ini
        m.vor2vel()
        te, en, _ = m.energy_series()
        m.init_diffusion(te, en)
        if use_net:
            attach(m, net, "every" in opts, "clip" in opts, "walls" in opts)
        ms, dt = cost_per_time(m, 0.0, 50)
        if use_net:
            attach(m, None)
        m.close()
        cost[f"{name}_ms_per_step"] = ms
        cost[f"{name}_dt"] = dt
    if timed:
        cost["timed_variant"] = timed[0][0]
        per_t_clos = cost["coarse_closure_ms_per_step"] / cost["coarse_closure_dt"]
        cost["closure_over_fine_mixed"] = per_t_clos / (ms_f / dt_f)
        if a.fp64_cost:
            cost["closure_over_fine_fp64"] = per_t_clos / (cost["fine_fp64_ms_per_step"] / cost["fine_fp64_dt"])

    final = {name: [e["variants"][name]["max_shell_error"][-1] if "max_shell_error" in e["variants"][name]
                    else None for e in evals] for name, _, _ in variants}
    out = {
        "workload": f"closure {nc}^3 trained on {nf}^3 ({a.precision}) Beltrami+perturbation runs",
        "fine": nf, "coarse": nc, "train_seeds": a.train_seeds, "test_seeds": a.test_seeds,
        "steps": a.steps, "sample_every": a.sample_every, "amplitude": a.amplitude,
        "samples": net.num_samples, "iters": a.iters, "variants": a.variants,
        "loss_first": float(loss[:20].mean()), "loss_last": float(loss[-50:].mean()),
        "ct": net.scale, "seconds": {"data": t_data, "train": t_train},
        "train_ms_per_iter": 1e3 * t_train / max(a.iters, 1),
        "final_max_shell_error": final,
        "evals": evals, "cost": cost,
    }
    print(json.dumps(out))


if __name__ == "__main__":
    main()
