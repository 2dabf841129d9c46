"""FP64 GPU path vs the oracle at the sizes the 512^3 accuracy figure and the
128^3 / 256^3 workloads rest on (the parity gate at full line lengths).

* Every FP64 field operator at line lengths 512 and 1024 in x and in y and
  column lengths 512 and 1024 in z (the FP64 line and column kernels pick
  other lane counts and radix schedules there than at the 8..64-point grids
  of test_gpu_parity.py), relative L2 within 1e-13.
* vor2vel (inversion.f90:23-226) and central_diffz (inversion_utils.f90:
  653-673) standalone at 128^3 and 256^3 on seeded random mixed-spectral
  vorticity with a K^(-5/3) amplitude spectrum and uniform random phases
  (ic.kolmogorov_spectral_vorticity): the projected svor, vor, vel and svel
  within 1e-12, the z derivative within 1e-13.
* 200 steps at 128^3 (Beltrami + perturbation, prediss 30, nnu 3, vorch,
  Kolmogorov, Hou & Li, CFL 0.5) with the per-step field L2 and the energy /
  enstrophy / helicity / dt series against the oracle; every one-step
  (local) error below 1e-13, and the trajectory error explained by those
  local errors (a shadow oracle run that receives them) (advance.f90:77-104).
"""
import numpy as np
import pytest

import oracle
from ps3d_gb300 import Ps3dGpu, ic
from tests.parity_util import multi_step_parity, rel_l2

pytestmark = pytest.mark.gpu

OP_TOL = 1.0e-13
FIELD_TOL = 1.0e-12
SERIES_TOL = 1.0e-10

LONG_GRIDS = [(512, 16, 8), (16, 512, 8), (1024, 8, 8), (8, 1024, 8), (8, 8, 512), (8, 8, 1024)]
OPS = ["fftxyp2s", "fftxys2p", "diffx", "diffy", "fftsine", "fftcosine", "central_diffz",
       "decompose_semi_spectral", "combine_semi_spectral", "decompose_physical", "combine_physical"]


@pytest.mark.parametrize("grid", LONG_GRIDS, ids=lambda g: "x".join(map(str, g)))
@pytest.mark.parametrize("op", OPS)
def test_fp64_operators_at_long_lines_match_oracle(grid, op):
    lo, ex = [0.0, -1.0, -0.25], [2 * np.pi, 3.0, 0.5 * np.pi]
    o = oracle.Oracle(*grid, lo, ex)
    g = Ps3dGpu(*grid, lo, ex)
    f = np.random.default_rng(21).standard_normal(o.shape)
    err = rel_l2(getattr(g, op)(f), getattr(o, op)(f))
    assert err < OP_TOL, (op, grid, err)


@pytest.mark.parametrize("n", [128, 256])
def test_standalone_vor2vel_and_diffz_on_kolmogorov_fields(n):
    lo, ex = ic.BELTRAMI_BOX["lower"], ic.BELTRAMI_BOX["extent"]
    svor = ic.kolmogorov_spectral_vorticity(n, n, n, ex, seed=100 + n)
    o = oracle.Oracle(n, n, n, lo, ex)
    g = Ps3dGpu(n, n, n, lo, ex)
    o.set("svor", svor)
    g.set("svor", svor)
    o.vor2vel()
    g.vor2vel()
    for name in ("svor", "vor", "vel", "svel"):
        a, b = g.get(name), o.get(name)
        for c in range(3):
            err = rel_l2(a[c], b[c])
            assert err < FIELD_TOL, (n, name, c, err)
    f = o.get("vor")[2]
    del a, b
    err = rel_l2(g.central_diffz(f), o.central_diffz(f))
    assert err < OP_TOL, (n, "central_diffz", err)


def test_200_steps_at_128_cubed_per_step_parity():
    """Per-step relative L2 of each vorticity component and the series over
    200 steps at 128^3 against the oracle (tests.parity_util.multi_step_parity):
    every local (one-step) error below 1e-13, the trajectory within 1e-12
    while the shadow run (the oracle carrying the GPU's local errors) is
    below 1e-13 and within 3x the shadow after.  The worst ratio of GPU error
    to shadow is printed."""
    ratio, at, series, eps = multi_step_parity(128, 200, check_every=10)
    print(f"128^3 x 200 steps: worst local (one-step) error {eps:.3g}; worst GPU/shadow ratio {ratio:.3g} at "
          f"(step, comp, err, floor) {at}; worst series error {series:.3g}")
