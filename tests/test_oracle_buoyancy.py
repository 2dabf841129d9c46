"""Pins of the oracle's buoyancy restatement (the reference built with
ENABLE_BUOYANCY).  The reference ships no unit test for this path, so the
restatement is checked against identities that hold to round-off:

* diffz (inversion_utils.f90:683-719) of fields the mixed-spectral form
  represents exactly (an interior sine mode, the harmonic functions, a
  linear profile in the (0,0) column);
* buoyancy_tendency (inversion.f90:232-292) under a uniform velocity, where
  -div(u b) - N^2 w is known in closed form;
* calculate_basic_reference_state (physics.f90:310-340) and the available
  potential energy (field_diagnostics.f90:29-60, ape_density.f90:10-34);
* conservation of kinetic + available potential energy by the inviscid
  Boussinesq steps (no hyperdiffusion).
"""
import numpy as np
import pytest

import oracle
from ps3d_gb300 import ic

BOX = ic.BELTRAMI_BOX


def _model(n=(16, 16, 16), lower=BOX["lower"], extent=BOX["extent"], **kw):
    kw.setdefault("buoyancy", True)
    return oracle.Oracle(*n, lower, extent, **kw)


@pytest.mark.parametrize("n", [(16, 16, 16), (16, 8, 32)])
def test_diffz_exact_modes(n):
    nx, ny, nz = n
    lo, ex = (0.0, -1.0, -0.3), (2 * np.pi, 2.0, 1.7)
    o = _model(n, lo, ex)
    x, y, z = ic.grid(nx, ny, nz, lo, ex)
    zz = z - lo[2]
    kx, ly = 2 * 2 * np.pi / ex[0], 1 * 2 * np.pi / ex[1]
    K = np.hypot(kx, ly)
    hor = np.cos(kx * x[:, None] + ly * y[None, :])
    m = 3 * np.pi / ex[2]
    # interior sine mode + both harmonic functions in one horizontal mode,
    # a linear profile in the (0, 0) column
    prof = (0.7 * np.sin(m * zz) + 1.3 * np.sinh(K * zz) / np.sinh(K * ex[2])
            - 0.4 * np.sinh(K * (ex[2] - zz)) / np.sinh(K * ex[2]))
    dprof = (0.7 * m * np.cos(m * zz) + 1.3 * K * np.cosh(K * zz) / np.sinh(K * ex[2])
             + 0.4 * K * np.cosh(K * (ex[2] - zz)) / np.sinh(K * ex[2]))
    f = hor[:, :, None] * prof[None, None, :] + (0.25 + 0.5 * z)[None, None, :]
    dfdz = hor[:, :, None] * dprof[None, None, :] + 0.5
    got = o.combine_physical(o.diffz(o.decompose_physical(f)))
    assert np.max(np.abs(got - dfdz)) < 1e-11 * np.max(np.abs(dfdz))


def test_diffz_requires_buoyancy_model():
    o = _model(buoyancy=False)
    with pytest.raises(ValueError):
        o.diffz(np.zeros(o.shape))


@pytest.mark.parametrize("bfsq", [0.0, 2.5])
def test_buoyancy_tendency_uniform_velocity(bfsq):
    """b_t = -(U b_x + V b_y + W b_z) - N^2 W for a uniform velocity."""
    n = (16, 16, 16)
    lo, ex = BOX["lower"], BOX["extent"]
    o = _model(n, lo, ex, bfsq=bfsq)
    x, y, z = ic.grid(*n, lo, ex)
    U, V, W = 0.3, -0.7, 0.45
    kx, ly, m = 2.0, 3.0, 2 * np.pi / ex[2]
    ph = kx * x[:, None] + ly * y[None, :]
    sz = np.sin(m * (z - lo[2]))
    cz = np.cos(m * (z - lo[2]))
    b = np.sin(ph)[:, :, None] * sz[None, None, :]
    bx = kx * np.cos(ph)[:, :, None] * sz[None, None, :]
    by = ly * np.cos(ph)[:, :, None] * sz[None, None, :]
    bz = m * np.sin(ph)[:, :, None] * cz[None, None, :]
    vel = np.stack([np.full(o.shape, U), np.full(o.shape, V), np.full(o.shape, W)])
    o.set("vel", vel)
    o.set("sbuoy", o.decompose_physical(b))
    o.buoyancy_tendency()
    got = o.combine_physical(o.get("sbuoys"))
    want = -(U * bx + V * by + W * bz) - bfsq * W
    assert np.max(np.abs(got - want)) < 1e-11 * np.max(np.abs(want))
    # the physical buoyancy of the step is left in buoy
    assert np.max(np.abs(o.get("buoy") - b)) < 1e-13


def test_basic_state_and_potential_energy():
    n = (16, 16, 16)
    lo, ex = BOX["lower"], BOX["extent"]
    bfsq = 1.7
    btot = ic.stratified_buoyancy(*n, lo, ex, bfsq=bfsq, amplitude=2e-2, seed=3)
    vor = ic.beltrami_vorticity(*n, lo, ex)
    o = _model(n, lo, ex)
    te, en = o.setup_fields(vor, buoy=btot)
    assert abs(o.bfsq - bfsq) < 1e-13 * bfsq
    x, y, z = ic.grid(*n, lo, ex)
    bp = btot - bfsq * z[None, None, :]
    assert np.max(np.abs(o.combine_physical(o.get("sbuoy")) - bp)) < 1e-12
    w = np.ones(n[2] + 1)
    w[0] = w[-1] = 0.5
    ape = np.sum(bp ** 2 / (2 * bfsq) * w) / (n[0] * n[1] * n[2])
    d = o.buoyancy_diagnostics()
    assert abs(d[0] - ape) < 1e-13 * ape
    ke = o.energy_series()[0]
    assert abs(te - (ke + ape)) < 1e-13 * te
    # N^2 given: the basic state is not recomputed
    o2 = _model(n, lo, ex, bfsq=0.5)
    o2.setup_fields(vor, buoy=btot)
    assert o2.bfsq == 0.5
    assert np.allclose(o2.table("bbarz"), 0.5 * z)


@pytest.mark.parametrize("stepper", ["impl-diff-rk4", "cn2"])
def test_inviscid_energy_conservation(stepper):
    """KE + APE is conserved by the inviscid Boussinesq equations.  Without
    hyperdiffusion the discrete steps keep the sum to the spatial truncation
    (it falls as n^-3: 1.3e-5, 1.6e-6, 2.1e-7 of E at 16^3, 32^3, 64^3 over
    t = 0.12, independent of dt), far below the exchange between the two
    (about 5% of E over the same time); a wrong sign in either coupling term
    would double the exchange instead of cancelling it."""
    n = (16, 16, 16)
    lo, ex = BOX["lower"], BOX["extent"]
    vor = 0.3 * ic.beltrami_vorticity(*n, lo, ex)
    btot = ic.stratified_buoyancy(*n, lo, ex, bfsq=4.0, amplitude=5e-2, seed=1, kmax=2)
    o = _model(n, lo, ex, stepper=stepper, prediss=0.0, buoy_prediss=0.0, pretype="constant",
               buoy_pretype="constant", filtering="2/3-rule", alpha=0.02, cflmax=0.2)
    o.setup_fields(vor, buoy=btot)
    o.vor2vel()

    def energy():
        ke = o.energy_series()[0]
        return ke + o.buoyancy_diagnostics()[0]

    e0, k0 = energy(), o.energy_series()[0]
    t = 0.0
    for _ in range(6):
        t, d = o.advance(t)
    o.vor2vel()
    e1, k1 = energy(), o.energy_series()[0]
    assert d["bfmax"] > 0.0 and d["bpref"] == 1.0
    assert abs(k1 - k0) > 1e-3 * e0
    assert abs(e1 - e0) < 1e-2 * abs(k1 - k0), (e0, e1, k0, k1)


def test_buoyancy_changes_the_trajectory():
    """With buoyancy the vorticity source gains (b_y, -b_x, 0)."""
    n = (16, 16, 16)
    lo, ex = BOX["lower"], BOX["extent"]
    vor, pert = ic.beltrami_plus_perturbation(*n, seed=2, amplitude=1e-3)
    btot = ic.stratified_buoyancy(*n, lo, ex, bfsq=1.0, amplitude=1e-2, seed=5)
    a = _model(n, lo, ex)
    b = _model(n, lo, ex, buoyancy=False)
    a.setup_fields(vor, pert, buoy=btot)
    b.setup_fields(vor, pert)
    a.vor2vel()
    b.vor2vel()
    a.source()
    b.source()
    # the difference of the sources is the buoyancy term, decomposed
    bp = a.get("buoy")
    bs = a.fftxyp2s(bp)
    dbx = a.decompose_semi_spectral(a.diffx(bs))
    dby = a.decompose_semi_spectral(a.diffy(bs))
    diff = a.get("svorts") - b.get("svorts")
    scale = np.max(np.abs(dby))
    assert np.max(np.abs(diff[0] - dby)) < 1e-10 * scale
    assert np.max(np.abs(diff[1] + dbx)) < 1e-10 * scale
    assert np.max(np.abs(diff[2])) < 1e-10 * scale
