"""Lengths with factors 3 and 5 (n = 2^a 3^b 5^c, the factorisation of
stafft.f90:128-187 with the radix-3 and radix-5 passes of :561-1017), GPU
against the oracle (which evaluates such lengths by the transform's
definition).

Both forms run these lengths through the shared-memory Stockham kernels with
radix-8/4/2/3/5 passes: FP64 operators within 1e-13, FP32 operators of the
mixed form within 2e-6, and a few whole steps at 48^3 and on a 40 x 30 x 24
grid (factors 5 and 3 in every direction).
"""
import numpy as np
import pytest

import oracle
from ps3d_gb300 import Ps3dGpu, ic
from tests.parity_util import rel_l2

pytestmark = pytest.mark.gpu

GRIDS = [(48, 8, 8), (8, 96, 8), (192, 16, 8), (8, 384, 8), (8, 8, 48), (8, 8, 96), (16, 8, 384), (40, 30, 24)]
OPS = ["fftxyp2s", "fftxys2p", "diffx", "diffy", "fftsine", "fftcosine", "decompose_semi_spectral",
       "combine_semi_spectral", "decompose_physical", "combine_physical"]


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-13), ("mixed", 2e-6)])
@pytest.mark.parametrize("grid", GRIDS, ids=lambda g: "x".join(map(str, g)))
@pytest.mark.parametrize("op", OPS)
def test_mixed_radix_operators_match_oracle(grid, op, precision, tol):
    lo, ex = [0.0, -1.0, -0.25], [2 * np.pi, 3.0, 0.5 * np.pi]
    o = oracle.Oracle(*grid, lo, ex)
    g = Ps3dGpu(*grid, lo, ex, precision=precision)
    f = np.random.default_rng(31).standard_normal(o.shape)
    err = rel_l2(getattr(g, op)(f), getattr(o, op)(f))
    assert err < tol, (op, grid, precision, err)


@pytest.mark.parametrize("grid", [(48, 48, 48), (40, 30, 24)], ids=lambda g: "x".join(map(str, g)))
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("mixed", 1e-6)])
def test_mixed_radix_steps_match_oracle(grid, precision, tol):
    nx, ny, nz = grid
    lo, ex = ic.BELTRAMI_BOX["lower"], ic.BELTRAMI_BOX["extent"]
    vor, pert = ic.beltrami_plus_perturbation(nx, ny, nz, seed=17, amplitude=1e-2)
    o = oracle.Oracle(nx, ny, nz, lo, ex, cflmax=0.5)
    g = Ps3dGpu(nx, ny, nz, lo, ex, cflmax=0.5, precision=precision)
    o.setup_fields(vor, pert)
    g.setup_fields(vor, pert)
    t_o = t_g = 0.0
    for _ in range(3):
        t_g, dg = g.advance(t_g)
        t_o, do = o.advance(t_o)
        assert abs(dg["ke"] - do["ke"]) <= tol * do["ke"]
    if precision == "mixed":
        o.vor2vel()
        g.vor2vel()
    err = rel_l2(g.get("svor"), o.get("svor"))
    assert err < tol, err
    assert abs(t_g - t_o) <= tol * t_o
