"""Benchmark of the ps3d hot path on GB300: Mpts*steps/s at 512^3.

One "step" is one advance() of the reference (vor2vel, adapt, source and an
impl-diff-rk4 step: four right-hand-side evaluations) on the 512^3 Beltrami
plus seeded-perturbation workload (prediss 30, nnu 3, vorch prefactor,
Kolmogorov viscosity, Hou & Li filter, CFL 0.5).  The headline value is the
mixed-precision form (FP32 transforms, products and stage arithmetic; FP64
prognostic vorticity, RK accumulators, low-mode inversion and reductions);
the plain FP64 form is timed beside it and the mixed form's relative L2
vorticity error against it is reported.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

After the headline the same workload runs once more at 1024^3 (mixed form
only; `large_grid` in the JSON line; --skip-large leaves it out).

With --impl reference the CPU restatement of the reference's algorithm
(oracle/, FP64, OpenMP over all host cores) is timed instead, one advance at
256^3 per step (a bounded sample of the same workload, reported per grid
point in the same unit).  Under torchrun every rank runs an independent
replica (the path does not shard across GPUs: replicas only, weak scaling).
"""
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


def log(*a):
    print(*a, file=sys.stderr, flush=True)


# ---------------------------------------------------------------- ranks
def dist_init(n_gpus):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws <= 1:
        return 0, 1, None
    import torch.distributed as dist
    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    dist.init_process_group("gloo")
    return dist.get_rank(), dist.get_world_size(), dist


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, v):
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# --------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi sampler for the timed region (SM clock, throttle reasons)."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                mx = float(f[1])
            except ValueError:
                continue
            for nm, v in zip(names, f[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------ workloads
def make_ic(n, seed=1):
    from ps3d_gb300 import ic
    if n >= 1024:  # 26 GB per vector field: build it slab by slab
        return ic.beltrami_plus_perturbation_slabs(n, n, n, seed=seed, amplitude=1.0e-3)
    return ic.beltrami_plus_perturbation(n, n, n, seed=seed, amplitude=1.0e-3)


def model_kw():
    return dict(nnu=3, prediss=30.0, pretype="vorch", length_scale="Kolmogorov",
                filtering="Hou & Li", stepper="impl-diff-rk4", cflmax=0.5, alpha=0.1)


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def fp64_peak_tflops(dev):
    """FP64 peak of this GPU as measured by a cuBLAS DGEMM through torch
    (plumbing: 2 n^3 flops per 4096^3 product, best of 5)."""
    try:
        import torch
        n = 4096
        a = torch.randn(n, n, dtype=torch.float64, device=f"cuda:{dev}")
        b = torch.randn(n, n, dtype=torch.float64, device=f"cuda:{dev}")
        torch.matmul(a, b)
        best = None
        for _ in range(5):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            torch.matmul(a, b)
            e1.record()
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1)
            best = ms if best is None else min(best, ms)
        del a, b
        torch.cuda.empty_cache()
        return 2.0 * n ** 3 / (best * 1e-3) / 1e12
    except Exception:
        return None


def cufft_comparator(n, dev):
    """cuFFT (torch.fft.rfft2 / irfft2 over x and y of an (n, n, P) FP32 field,
    z contiguous as here) timed as a comparator for one forward and one
    inverse horizontal transform."""
    try:
        import torch
        P = (n + 1 + 7) // 8 * 8
        x = torch.randn(n, n, P, dtype=torch.float32, device=f"cuda:{dev}")
        def t(fn, reps=5):
            fn()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(reps):
                out = fn()
            e1.record()
            torch.cuda.synchronize()
            return e0.elapsed_time(e1) / reps, out
        fwd_ms, X = t(lambda: torch.fft.rfft2(x, dim=(0, 1)))
        inv_ms, _ = t(lambda: torch.fft.irfft2(X, s=(n, n), dim=(0, 1)))
        del x, X
        torch.cuda.empty_cache()
        return {"forward_xy_ms": fwd_ms, "inverse_xy_ms": inv_ms,
                "how": "torch.fft.rfft2 / irfft2 (cuFFT) over dims 0, 1 of an (n, n, P) float32 field"}
    except Exception as e:
        return {"unavailable": str(e)[:200]}


def closure_timing(dev, n=64):
    """The learned closure's forward pass (four BF16 tensor-core 3x3x3
    convolutions, closure.cu) at n^3 against the measured bf16 peak, and its
    cost inside a coarse step: one captured impl-diff-rk4 advance at n^3 with
    and without a network evaluated at every stage, each also per unit of
    model time against the fine (4n)^3 mixed run (the closure's bar: 1/20)."""
    try:
        from ps3d_gb300 import Ps3dGpu, ic
        from ps3d_gb300.closure import Closure, attach, forward_flops, param_views
        cl = Closure(n, n, n, device=dev, seed=3)
        p = cl.get_params()
        param_views(p)[-1][0][...] *= 10.0
        cl.set_params(p)
        cl.scale = 1e-3
        rng = np.random.default_rng(0)
        shape = (3, n, n, n + 1)
        vr, ur = rng.standard_normal(shape), rng.standard_normal(shape)
        engines = {}
        for eng in ("mma", "tcgen05"):
            try:
                cl.engine = eng
                cl.predict(vr, ur)
                engines[eng] = cl.time_forward(50)
                cl.check()
            except Exception as e:  # an engine the grid does not support
                engines[eng] = None
                log(f"[bench] closure engine {eng}: {e}")
        best = min((v, k) for k, v in engines.items() if v is not None)
        ms, eng_best = best
        cl.engine = eng_best
        npts = n * n * (n + 1)
        tf = forward_flops(npts) / (ms * 1e9)
        try:
            with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
                pk, src = float(json.load(f)["bf16_tflops"]), "measured (MEASURED_PEAKS.json bf16_tflops)"
        except (OSError, KeyError, ValueError):
            pk, src = 1900.0, "fallback"
        def timed_run(nn, net=None):
            # 20 captured advances after 3; ms per step and the mean dt
            vv, pp = ic.beltrami_plus_perturbation(nn, nn, nn, seed=1, amplitude=1.0e-2)
            m = Ps3dGpu(nn, nn, nn, ic.BELTRAMI_BOX["lower"], ic.BELTRAMI_BOX["extent"], precision="mixed",
                        device=dev, **model_kw())
            m.setup_fields(vv, pp)
            if net is not None:
                attach(m, net, every_stage=True)
            t0, _, _ = m.advance_graph(0.0, 3)
            t1, _, mss = m.advance_graph(t0, 20)
            if net is not None:
                attach(m, None)
            m.close()
            return mss / 20, (t1 - t0) / 20
        steps, dts = {}, {}
        for name, net in (("plain", None), ("closure_every_stage", cl)):
            steps[name], dts[name] = timed_run(n, net)
        cl.close()
        # the cost of a unit of model time against the fine (4n)^3 run of the
        # mixed form that the closure stands in for
        nf = 4 * n
        fine_ms, fine_dt = timed_run(nf)
        per_time = {k: (steps[k] / dts[k]) / (fine_ms / fine_dt) for k in steps}
        return {"grid": [n, n, n], "engine": eng_best, "ms_per_forward_by_engine": engines,
                "ms_per_forward": ms, "flops_per_forward": forward_flops(npts),
                "roofline": {"bound": "tensor", "achieved": tf, "peak": pk, "unit": "TFLOP/s", "frac": tf / pk,
                             "peak_source": src},
                "tflops_padded_channels": forward_flops(npts, True) / (ms * 1e9),
                "step_ms": steps, "mean_dt": dts,
                "fine_mixed": {"grid": [nf, nf, nf], "ms_per_step": fine_ms, "mean_dt": fine_dt},
                "cost_per_model_time_vs_fine_mixed": per_time}
    except Exception as e:
        return {"unavailable": str(e)[:200]}


def batch_timing(steps, warmup=3):
    """The batched workload: 96 independent runs of uneven sizes (48 x 32^3,
    32 x 64^3, 16 x 128^3), each Beltrami plus its own seeded perturbation
    (amplitude log-uniform in [1e-4, 1e-2]) and prediss from {10, 30, 60,
    90}, mixed form; every batch step is one CUDA graph with one persistent
    launch per stage update for all runs (ps3d_gpu_batch_advance)."""
    try:
        from ps3d_gb300 import batch_advance, batch_case
        counts = [(32, 48), (64, 32), (128, 16)]
        runs = batch_case.build(counts, seed=7)
        models = [r[3] for r in runs]
        pts = sum(n ** 3 for n, _, _, _ in runs)
        ts = [0.0] * len(models)
        ts, _ = batch_advance(models, ts, warmup)
        ts, ms = batch_advance(models, ts, steps)
        out = {"runs": len(models), "counts": {f"{n}^3": c for n, c in counts}, "points_per_step": pts,
               "steps": steps, "ms_per_step": ms / steps, "value": pts * steps / (ms * 1e-3) / 1e6,
               "unit": "Mpts*steps/s",
               "how": "one CUDA graph per batch step; one persistent stage-update launch per RK stage"}
        for m in models:
            m.close()
        return out
    except Exception as e:
        return {"unavailable": str(e)[:200]}


def cpu_sample(n_cpu, steps=1):
    """Time the CPU oracle: `steps` advances at n_cpu^3 after one warm-up."""
    import oracle
    from ps3d_gb300 import ic
    vor, pert = make_ic(n_cpu)
    o = oracle.Oracle(n_cpu, n_cpu, n_cpu, ic.BELTRAMI_BOX["lower"], ic.BELTRAMI_BOX["extent"], **model_kw())
    o.setup_fields(vor, pert)
    t = 0.0
    t, _ = o.advance(t)
    t0 = time.perf_counter()
    for _ in range(steps):
        t, _ = o.advance(t)
    sec = (time.perf_counter() - t0) / steps
    return sec, n_cpu ** 3 / sec / 1e6


def run_reference(args, rank, world, dist):
    """--impl reference: the reference's algorithm on the host cores."""
    if rank != 0:
        return
    import oracle
    from ps3d_gb300 import ic
    n = args.cpu_n
    cores = os.cpu_count()
    vor, pert = make_ic(n)
    o = oracle.Oracle(n, n, n, ic.BELTRAMI_BOX["lower"], ic.BELTRAMI_BOX["extent"], nthreads=cores,
                      **model_kw())
    o.setup_fields(vor, pert)
    t = 0.0
    for _ in range(args.warmup):
        t, _ = o.advance(t)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        t, _ = o.advance(t)
    sec = time.perf_counter() - t0
    value = n ** 3 * args.steps / sec / 1e6
    sample = f"{args.steps} advance() steps of the FP64 oracle at {n}^3 (same workload, per-point rate)"
    line = {
        "impl": "reference", "metric": "Mpts*steps/s", "value": value, "unit": "Mpts*steps/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * sec / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"beltrami+perturbation {args.n}^3 impl-diff-rk4 (sampled at {n}^3 on CPU)",
                   "grid": [args.n] * 3, "sample_grid": [n] * 3, "parallelism": "replicas"},
        "cpu_baseline": {"value": value, "unit": "Mpts*steps/s", "cores": cores, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": "Mpts*steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_gpu(args, rank, world, dist):
    from ps3d_gb300 import Ps3dGpu, ic
    n = args.n
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    pts = float(n) ** 3
    lower, extent = ic.BELTRAMI_BOX["lower"], ic.BELTRAMI_BOX["extent"]
    t_ic = time.perf_counter()
    vor, pert = make_ic(n, seed=1 + rank)
    log(f"[bench] rank {rank}: IC {n}^3 in {time.perf_counter() - t_ic:.1f}s")

    # ---- mixed precision (headline) ----------------------------------
    gm = Ps3dGpu(n, n, n, lower, extent, precision="mixed", device=dev, **model_kw())
    gm.setup_fields(vor, pert)
    t_m = 0.0
    # warm-up: host-driven steps, then one captured step (builds the graph)
    for _ in range(max(args.warmup - 1, 1)):
        t_m, _ = gm.advance(t_m)
    t_m, _, _ = gm.advance_graph(t_m, 1)
    gm.synchronize()
    launches0 = gm.launch_count
    barrier(dist)
    with ClockSampler(dev) as clk:
        # every step one CUDA graph launch (same arithmetic as advance())
        t_m, _, ms = gm.advance_graph(t_m, args.steps)
    barrier(dist)
    launches = gm.launch_count - launches0
    sec = max_over_ranks(dist, ms / 1e3)
    value = world * pts * args.steps / sec / 1e6
    clocks = clk.summary()

    # dominant kernel probe inside real steps (same stream, CUDA events).
    # k_lines32 (the line FFT, both directions), the k_colz column-kernel
    # family and the source's products-plus-forward-y-lines kernel are the
    # candidates; y and x lines are also reported apart.
    probe_steps = max(1, min(3, args.steps))
    best = None
    probes = []
    kinds = ((4, "k_lines32 (x and y lines)", True), (3, "k_colz (column transforms)", True),
             (1, "k_lines32 (y lines)", False), (2, "k_lines32 (x lines)", False),
             (5, "k_lines32_prod (source products + forward y lines)", True))
    for kind, name, candidate in kinds:
        gm.probe(kind)
        t_m, _ = gm.time_advance(t_m, probe_steps)
        kms, nl, kbytes = gm.probe_result()
        gm.probe(0)
        share = kms / (ms / args.steps * probe_steps) if ms > 0 else 0.0
        rec = {"kernel": name, "launches_per_step": nl / probe_steps, "ms_per_launch": kms / max(nl, 1),
               "bytes_per_launch": kbytes / max(nl, 1), "share_of_step": share}
        probes.append(rec)
        if candidate and (best is None or kms > best[1]):
            best = (rec, kms, kind)
    peak, peak_kind = peaks()
    krec = best[0]
    achieved = krec["bytes_per_launch"] / (krec["ms_per_launch"] * 1e-3) / 1e9
    # DRAM traffic of the line kernels per field pass: ncu read + write bytes
    # of the plain line launches of one 512 x 512 x 128 advance (21.0 GB over
    # 78 field passes, 269.3 MB each; profiles/step_traffic_512x512x128.md),
    # scaled to 512^3
    # by the field size ratio P(512) / P(128) = 520 / 136 (traffic grows with
    # the column pitch at fixed nx, ny), times the field passes per launch (a
    # launch transforms up to five fields); not measured for other kernels or
    # sizes
    traffic = None
    if best[2] == 4 and n == 512:
        field_pass = 2.0 * n * n * (n + 1) * 4.0
        traffic = 269.3e6 * 520.0 / 136.0 * (krec["bytes_per_launch"] / field_pass)
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": traffic, "traffic_unit": "bytes per launch",
                "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of the line launches of one "
                                  "512x512x128 advance, per field pass, scaled by 520/136 and by the field "
                                  "passes per launch (profiles/k_lines32_512.md)"
                if traffic else None,
                "kernel": krec["kernel"],
                "algorithmic_bytes_per_launch": krec["bytes_per_launch"],
                "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else peak_kind,
                "kernel_share_of_step": krec["share_of_step"],
                "probes": probes}
    svor_mixed_steps = args.warmup + args.steps + len(kinds) * probe_steps

    # ---- FP64 form: timing, and the reference for the mixed error --------
    # Both forms run the same `accuracy_steps` advances from the same state;
    # the FP64 throughput is timed over all of them.
    fp64 = None
    if not args.skip_fp64:
        nacc = max(args.accuracy_steps, svor_mixed_steps)
        if nacc > svor_mixed_steps:
            t_m, _ = gm.advance_n(t_m, nacc - svor_mixed_steps)
        g64 = Ps3dGpu(n, n, n, lower, extent, precision="fp64", device=dev, **model_kw())
        g64.setup_fields(vor, pert)
        t64, ms64 = g64.time_advance(0.0, nacc)
        sec64 = max_over_ranks(dist, ms64 / 1e3)
        # solenoidal states (the FP64 form projects svor in vor2vel)
        g64.vor2vel()
        gm.vor2vel()
        a = gm.get("svor")
        b = g64.get("svor")
        err = float(np.linalg.norm(a - b) / np.linalg.norm(b))
        v64 = world * pts * nacc / sec64 / 1e6
        fp64 = {"value": v64, "unit": "Mpts*steps/s", "ms_per_step": 1e3 * sec64 / nacc,
                "steps": nacc, "mixed_speedup": value / v64,
                "mixed_rel_l2_vs_fp64": err, "after_steps": nacc, "bar": 1.0e-6,
                "t_mixed": t_m, "t_fp64": t64}
        del a, b
        g64.close()

    # ---- end to end through the public API with host buffers ------------
    e2e = None
    if not args.skip_e2e:
        host, host_kind, host_owner = pinned_like((3, n, n, n + 1))
        host[...] = gm.get("svor")
        nb = host.nbytes
        e2e_steps = max(1, min(args.steps, 5))
        t_e = t_m
        t_e, _ = gm.advance_host(host, t_e)   # warm
        barrier(dist)
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            t_e, _ = gm.advance_host(host, t_e)
        esec = max_over_ranks(dist, time.perf_counter() - t0)
        e2e = {"value": world * pts * e2e_steps / esec / 1e6, "unit": "Mpts*steps/s",
               "h2d_bytes_per_step": nb, "d2h_bytes_per_step": nb, "steps": e2e_steps,
               "api": "ps3d_gpu_advance_host (svor FP64 in/out)", "host_buffer": host_kind}

    # FP64 form against the FP64 ALU roofline (flop model: 49 transforms per
    # impl-diff-rk4 step at 2.5 N log2 n each, plus ~300 flop per point for
    # the strain eigen-solve) and cuFFT as a comparator for the horizontal
    # transforms
    if fp64 is not None:
        pk = fp64_peak_tflops(dev)
        N = float(n) ** 2 * (n + 1)
        flops = 49 * 2.5 * N * (3 * np.log2(n)) + 300.0 * N
        ach = flops / (fp64["ms_per_step"] * 1e-3) / 1e12
        fp64["alu"] = {"flops_per_step": flops, "achieved_tflops": ach, "peak_tflops": pk,
                       "frac": (ach / pk) if pk else None,
                       "peak_source": "cuBLAS DGEMM 4096^3 through torch, best of 5"}
    cufft = None
    if rank == 0:
        cufft = cufft_comparator(n, dev)
        # our time per field for one y pass plus one x pass (a launch may
        # transform several fields: time per launch over field passes)
        fp_bytes = 2.0 * n * n * (n + 1) * 4.0
        lp = {p["kernel"]: p["ms_per_launch"] * fp_bytes / max(p["bytes_per_launch"], 1.0)
              for p in roofline["probes"]}
        ours = lp.get("k_lines32 (y lines)", 0.0) + lp.get("k_lines32 (x lines)", 0.0)
        if isinstance(cufft, dict) and "forward_xy_ms" in cufft:
            cufft["ours_xy_pass_pair_ms"] = ours

    closure = closure_timing(dev) if rank == 0 and not args.skip_closure else None
    batch = batch_timing(args.batch_steps) if rank == 0 and not args.skip_batch else None
    device_bytes, tuning = gm.device_bytes, dict(zip(("shape", "ms_per_launch"), gm.tuning()))

    cpu = None
    if rank == 0 and not args.skip_cpu:
        csec, crate = cpu_sample(args.cpu_n)
        cpu = {"value": crate, "unit": "Mpts*steps/s", "cores": os.cpu_count(), "kind": "port",
               "sample": f"1 advance() at {args.cpu_n}^3 (FP64 oracle, OpenMP), {csec:.2f} s"}

    if rank == 0:
        line = {
            "metric": "Mpts*steps/s", "value": value, "unit": "Mpts*steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sec / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 transforms / f64 state (mixed)", "data": "synthetic",
            "config": {"workload": f"beltrami+perturbation {n}^3 impl-diff-rk4 advance (mixed precision)",
                       "grid": [n, n, n], "stepper": "impl-diff-rk4", "prediss": 30, "nnu": 3,
                       "cfl": 0.5, "parallelism": "replicas" if world > 1 else "single",
                       "l2": "inputs larger than L2 (each field >= 0.5 GB)",
                       "timed_steps": "graph-captured (ps3d_gpu_advance_graph)"},
            "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "fp64": fp64,
            "gpu_launches": launches, "clocks": clocks,
            "device_bytes": device_bytes,
            "line_fft_autotune": tuning,
            "cufft_comparator": cufft,
            "closure": closure,
            "batch": batch,
        }
    gm.close()
    if rank == 0:
        line["large_grid"] = None if args.skip_large or n >= args.large_n else large_grid_timing(args, dev)
        print(json.dumps(line), flush=True)


def large_grid_timing(args, dev):
    """The mixed form at large_n^3 (1024^3: the context holds ~225 GB of the
    GPU's HBM), the same workload with the perturbation built slab by slab
    on the host; graph-captured steps timed with CUDA events after
    `warmup` steps, as the headline.  Runs after every other context is
    closed."""
    from ps3d_gb300 import Ps3dGpu, ic
    try:
        import torch
        torch.cuda.empty_cache()
    except Exception:
        pass
    n = args.large_n
    t0 = time.perf_counter()
    vor, pert = make_ic(n, seed=1)
    t_ic = time.perf_counter() - t0
    try:
        g = Ps3dGpu(n, n, n, ic.BELTRAMI_BOX["lower"], ic.BELTRAMI_BOX["extent"], precision="mixed", device=dev,
                    **model_kw())
    except Exception as e:  # not enough device memory on this GPU
        return {"grid": [n, n, n], "skipped": str(e)[:200]}
    try:
        g.setup_fields(vor, pert)
        del vor, pert
        t = 0.0
        for _ in range(max(args.warmup - 1, 1)):
            t, _ = g.advance(t)
        t, _, _ = g.advance_graph(t, 1)
        g.synchronize()
        with ClockSampler(dev) as clk:
            t, _, ms = g.advance_graph(t, args.large_steps)
        ms_step = ms / args.large_steps
        return {"grid": [n, n, n], "value": float(n) ** 3 / (ms_step * 1e-3) / 1e6, "unit": "Mpts*steps/s",
                "ms_per_step": ms_step, "steps": args.large_steps, "warmup": args.warmup,
                "device_bytes": g.device_bytes, "clocks": clk.summary(), "ic_seconds": t_ic,
                "timed_steps": "graph-captured (ps3d_gpu_advance_graph)"}
    finally:
        g.close()


def pinned_like(shape):
    """Page-locked host array: from the library (ps3d_gpu_host_alloc), else a
    pinned torch tensor viewed through numpy, else cudaHostAlloc through
    libcudart, else pageable.  Returns (array, how, owner); keep owner alive with the array."""
    try:
        from ps3d_gb300.solver import PinnedArray
        pa = PinnedArray(shape)
        return pa.array, "ps3d_gpu_host_alloc", pa
    except Exception:
        pass
    try:
        import torch
        t = torch.empty(tuple(shape), dtype=torch.float64, pin_memory=True)
        return t.numpy(), "torch.pin_memory", t
    except Exception:
        pass
    import ctypes
    nbytes = int(np.prod(shape)) * 8
    for name in ("libcudart.so", "libcudart.so.13", "/usr/local/cuda/lib64/libcudart.so"):
        try:
            rt = ctypes.CDLL(name)
            break
        except OSError:
            rt = None
    if rt is not None:
        p = ctypes.c_void_p()
        if rt.cudaHostAlloc(ctypes.byref(p), ctypes.c_size_t(nbytes), 0) == 0:
            buf = (ctypes.c_double * (nbytes // 8)).from_address(p.value)
            return np.frombuffer(buf, dtype=np.float64).reshape(shape), "cudaHostAlloc", buf
    return np.empty(shape), "pageable", None


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--n", type=int, default=512)
    ap.add_argument("--cpu-n", type=int, default=256)
    ap.add_argument("--accuracy-steps", type=int, default=100)
    ap.add_argument("--skip-fp64", action="store_true")
    ap.add_argument("--skip-e2e", action="store_true")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-closure", action="store_true")
    ap.add_argument("--skip-batch", action="store_true")
    ap.add_argument("--batch-steps", type=int, default=500)
    ap.add_argument("--skip-large", action="store_true")
    ap.add_argument("--large-n", type=int, default=1024)
    ap.add_argument("--large-steps", type=int, default=3)
    args = ap.parse_args()
    if args.warmup < 3:
        log("[bench] warm-up raised to 3 steps")
        args.warmup = 3
    rank, world, dist = dist_init(args.gpus)
    if args.impl == "reference":
        run_reference(args, rank, world, dist)
    else:
        run_gpu(args, rank, world, dist)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
