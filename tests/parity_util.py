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


def multi_step_parity(n, nsteps, check_every, field_tol=1.0e-12, series_tol=1.0e-10, seed=1):
    """GPU (FP64 form) against the oracle over nsteps advances of the n^3
    Beltrami + perturbation run (prediss 30, nnu 3, vorch, CFL 0.5), with
    the per-step relative L2 of each vorticity component and the energy /
    enstrophy / helicity / dt series.

    The perturbed Beltrami state is unstable, so any rounding-level
    difference grows over the run whatever produced it.  The rounding floor
    is a second oracle run that differs from the first by rounding-sized
    noise at every step: after each advance its state is multiplied
    element-wise by (1 + eps g), g standard normal, eps the GPU's own
    one-step relative difference from the oracle (itself required below
    1e-13, so a wrong step cannot widen the floor).  The GPU must stay
    within field_tol of the oracle while the floor is below field_tol / 10
    and within 10x the floor after.  Returns (worst GPU/floor ratio, where,
    worst series error, eps)."""
    from ps3d_gb300 import Ps3dGpu as _G
    lo, ex, vor, pert = beltrami_case(n, seed=seed)
    o = oracle.Oracle(n, n, n, lo, ex, cflmax=0.5)
    f = oracle.Oracle(n, n, n, lo, ex, cflmax=0.5)
    g = _G(n, n, n, lo, ex, cflmax=0.5)
    for m in (o, f, g):
        m.setup_fields(vor, pert)
    rng = np.random.default_rng(5)
    t_o = t_g = t_f = 0.0
    worst_series, worst_ratio, worst_at, eps = 0.0, 0.0, None, None
    for s in range(nsteps):
        t_g, dg = g.advance(t_g)
        t_o, do = o.advance(t_o)
        t_f, _ = f.advance(t_f)
        if eps is None:
            a, b = g.get("svor"), o.get("svor")
            eps = max(rel_l2(a[c], b[c]) for c in range(3))
            assert eps < 1.0e-13, ("one-step difference", eps)
            eps = max(eps, 1.0e-16)
        sv = f.get("svor")
        f.set("svor", sv * (1.0 + eps * rng.standard_normal(sv.shape)))
        for k in ("ke", "en", "hel", "dt"):
            worst_series = max(worst_series, abs(dg[k] - do[k]) / abs(do[k]))
        if s % check_every == 0 or s == nsteps - 1:
            a, b, c_ = g.get("svor"), o.get("svor"), f.get("svor")
            for c in range(3):
                err = rel_l2(a[c], b[c])
                floor = rel_l2(c_[c], b[c])
                bound = field_tol if floor < 0.1 * field_tol else 10.0 * floor
                assert err < bound, (s, c, err, floor)
                if floor > 0 and err / floor > worst_ratio:
                    worst_ratio, worst_at = err / floor, (s, c, err, floor)
    assert worst_series < series_tol, worst_series
    assert abs(t_g - t_o) <= 1e-10 * t_o
    return worst_ratio, worst_at, worst_series, eps
