"""Small, self-contained workload for timing and profiling the closure's
convolution kernels (closure.cu) with ncu.

    python -m ps3d_gb300.profile_closure --n 128 --reps 3

Builds a closure network for an n^3 grid (engine mma or tcgen05) (n x n x (n+1) points), runs one
forward pass on seeded random vorticity and velocity (predict), then `reps`
timed forward passes, and prints one JSON line: ms per forward pass and the
tensor throughput in TFLOP/s (multiply-adds of the real channel counts, and
of the padded counts the kernels compute with).
"""
import argparse
import json

import numpy as np

from .closure import Closure, forward_flops, param_views


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=64)
    ap.add_argument("--reps", type=int, default=20)
    ap.add_argument("--engine", default="mma", choices=["mma", "tcgen05"])
    a = ap.parse_args(argv)
    n = a.n
    cl = Closure(n, n, n, seed=3)
    p = cl.get_params()
    param_views(p)[-1][0][...] *= 10.0
    cl.set_params(p)
    cl.scale = 1.0
    cl.engine = a.engine
    rng = np.random.default_rng(0)
    shape = (3, n, n, n + 1)
    cl.predict(rng.standard_normal(shape), rng.standard_normal(shape))
    ms = cl.time_forward(a.reps)
    npts = n * n * (n + 1)
    kern = "k_conv_tc (4 layers)" if a.engine == "tcgen05" else "k_conv (4 layers)"
    out = {"kernel": kern, "engine": a.engine, "grid": [n, n, n], "points": npts, "reps": a.reps,
           "ms_per_forward": ms, "tflops": forward_flops(npts) / (ms * 1e9),
           "tflops_padded": forward_flops(npts, True) / (ms * 1e9)}
    print(json.dumps(out))
    cl.close()


if __name__ == "__main__":
    main()
