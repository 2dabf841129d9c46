"""Small, self-contained workload for profiling one kernel class with ncu.

    python -m ps3d_gb300.profile_case --n 256 --precision mixed --steps 1

Sets up the Beltrami plus perturbation field at n^3, runs `warmup` advances
and then `steps` advances (the launches to capture), and prints the device
time per advance.  Keeps the device footprint to a few GB at n <= 256.
"""
import argparse
import sys

from . import Ps3dGpu, ic


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=256)
    ap.add_argument("--nx", type=int, default=0)
    ap.add_argument("--ny", type=int, default=0)
    ap.add_argument("--nz", type=int, default=0)
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--steps", type=int, default=1)
    ap.add_argument("--warmup", type=int, default=1)
    a = ap.parse_args(argv)
    nx, ny, nz = a.nx or a.n, a.ny or a.n, a.nz or a.n
    vor, pert = ic.beltrami_plus_perturbation(nx, ny, nz, seed=1)
    g = Ps3dGpu(nx, ny, nz, ic.BELTRAMI_BOX["lower"], ic.BELTRAMI_BOX["extent"], precision=a.precision,
                nnu=3, prediss=30.0, pretype="vorch", cflmax=0.5)
    g.setup_fields(vor, pert)
    t = 0.0
    if a.warmup:
        t, _ = g.advance_n(t, a.warmup)
    t, ms = g.time_advance(t, a.steps)
    print(f"profile_case {nx}x{ny}x{nz} {a.precision}: {ms / max(a.steps, 1):.3f} ms/advance, "
          f"{g.launch_count} launches total", file=sys.stderr)
    g.close()


if __name__ == "__main__":
    main()
