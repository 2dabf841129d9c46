"""Helpers shared by the GPU parity tests (GPU library vs CPU oracle)."""
import numpy as np

import oracle
from ps3d_gb300 import Ps3dGpu, ic


def rel_l2(a, b):
    den = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (den if den > 0 else 1.0))


def pair(nx, ny, nz, lower, extent, precision="fp64", **kw):
    o = oracle.Oracle(nx, ny, nz, lower, extent, **kw)
    g = Ps3dGpu(nx, ny, nz, lower, extent, precision=precision, **kw)
    return o, g


def beltrami_case(n, seed=1, amplitude=1.0e-3, **kw):
    lower, extent = ic.BELTRAMI_BOX["lower"], ic.BELTRAMI_BOX["extent"]
    vor, pert = ic.beltrami_plus_perturbation(n, n, n, seed=seed, amplitude=amplitude)
    return lower, extent, vor, pert


def random_field(shape, seed):
    return np.random.default_rng(seed).standard_normal(shape)
