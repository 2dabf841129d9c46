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


def multi_step_parity(n, nsteps, check_every, field_tol=1.0e-12, local_tol=1.0e-13, series_tol=1.0e-10, seed=1):
    """GPU (FP64 form) against the oracle over nsteps advances of the n^3
    Beltrami + perturbation run (prediss 30, nnu 3, vorch, CFL 0.5), with
    the per-step relative L2 of each vorticity component and the energy /
    enstrophy / helicity / dt series.

    The perturbed Beltrami state is unstable, so any rounding-level
    difference grows over the run whatever produced it.  Two things are
    checked at every step:
    * the local error: a second GPU context advanced one step from the
      oracle's own state differs from the oracle's step by less than
      local_tol (the one-step parity bar, relative L2);
    * the trajectory: a shadow oracle run receives, after each of its
      steps, exactly that local error field, so it carries the GPU's
      rounding differences through the oracle's own dynamics.  The GPU run
      must stay within field_tol of the oracle while the shadow is below
      field_tol / 10, and within 3x the shadow's distance after (to first
      order the two are equal: the GPU's divergence is its local errors,
      amplified by the flow).
    Returns (worst GPU/shadow ratio, where, worst series error, worst
    local error)."""
    from ps3d_gb300 import Ps3dGpu as _G
    lo, ex, vor, pert = beltrami_case(n, seed=seed)
    o = oracle.Oracle(n, n, n, lo, ex, cflmax=0.5)
    f = oracle.Oracle(n, n, n, lo, ex, cflmax=0.5)
    g = _G(n, n, n, lo, ex, cflmax=0.5)
    h = _G(n, n, n, lo, ex, cflmax=0.5)
    for m in (o, f, g, h):
        m.setup_fields(vor, pert)
    # the shadow starts from the GPU's own set-up state (its rounding of the
    # initial decomposition is part of what it carries)
    f.set("svor", g.get("svor"))
    t_o = t_g = t_f = 0.0
    worst_series, worst_ratio, worst_at, worst_local = 0.0, 0.0, None, 0.0
    for s in range(nsteps):
        h.set("svor", o.get("svor"))
        h.advance(t_o)
        t_g, dg = g.advance(t_g)
        t_o, do = o.advance(t_o)
        t_f, _ = f.advance(t_f)
        so = o.get("svor")
        e = h.get("svor") - so
        local = max(rel_l2(e[c] + so[c], so[c]) for c in range(3))
        assert local < local_tol, ("local error", s, local)
        worst_local = max(worst_local, local)
        f.set("svor", f.get("svor") + e)
        for k in ("ke", "en", "hel", "dt"):
            worst_series = max(worst_series, abs(dg[k] - do[k]) / abs(do[k]))
        if s % check_every == 0 or s == nsteps - 1:
            a, c_ = g.get("svor"), f.get("svor")
            for c in range(3):
                err = rel_l2(a[c], so[c])
                floor = rel_l2(c_[c], so[c])
                bound = field_tol if floor < 0.1 * field_tol else 3.0 * floor
                assert err < bound, (s, c, err, floor)
                if floor > 0 and err / floor > worst_ratio:
                    worst_ratio, worst_at = err / floor, (s, c, err, floor)
    assert worst_series < series_tol, worst_series
    assert abs(t_g - t_o) <= 1e-10 * t_o
    return worst_ratio, worst_at, worst_series, worst_local
