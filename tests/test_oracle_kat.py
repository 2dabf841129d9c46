"""Pin the CPU oracle against the reference's own known-answer unit tests.

Every case here is a port of a program in the reference's unit-tests/
directory; each runs on the oracle with the grid, box and tolerance the
reference program uses.  These are the golden vectors of the path: the
reference ships no recorded outputs and cannot be built here.
"""
import numpy as np
import pytest

import oracle
from tests import kat_cases as K


def _model(c, **kw):
    return oracle.Oracle(c["nx"], c["ny"], c["nz"], c["lower"], c["extent"], **kw)


@pytest.mark.parametrize("name", sorted(K.VOR2VEL_CASES))
def test_vor2vel_known_answer(name):
    """unit-tests/test_vor2vel_{1..5}.f90: decompose the analytic vorticity,
    run vor2vel, compare the velocity with the analytic one (max-abs)."""
    c = K.VOR2VEL_CASES[name]()
    m = _model(c)
    svor = np.stack([m.decompose_physical(c["vor"][i]) for i in range(3)])
    m.set("svor", svor)
    m.vor2vel()
    err = np.abs(m.get("vel") - c["vel"]).max()
    assert err < c["atol"], (name, err)


@pytest.mark.parametrize("name", ["diffz_1", "diffz_2", "diffz_3", "diffz_4"])
def test_central_diffz_known_answer(name):
    c = K.diffz_cases()[name]
    m = _model(c)
    err = np.abs(m.central_diffz(c["f"]) - c["dfdz"]).max()
    assert err < c["atol"], (name, err)


@pytest.mark.parametrize("name", ["diffx", "diffy"])
def test_diffxy_known_answer(name):
    """unit-tests/test_diffx.f90 / test_diffy.f90: fftxyp2s, diffx|diffy,
    fftxys2p on cos(4x) / cos(4y)."""
    c = K.diffxy_cases()[name]
    m = _model(c)
    fs = m.fftxyp2s(c["f"])
    ds = m.diffx(fs) if c["axis"] == "x" else m.diffy(fs)
    fp = m.fftxys2p(ds)
    err = np.abs(fp - c["df"]).max()
    assert err < c["atol"], (name, err)


def test_omp_collapse_dst_deterministic():
    """unit-tests/test_omp_collapse.f90: the column DST of the decomposed
    Beltrami velocity is the same whichever way the column loop is split."""
    lower, extent = [-0.5 * np.pi] * 3, [np.pi] * 3
    vor, vel = K.beltrami(64, 64, 64, lower, extent)
    m1 = oracle.Oracle(64, 64, 64, lower, extent, nthreads=1)
    svel = np.stack([m1.decompose_physical(vel[i]) for i in range(3)])
    a = np.stack([m1.fftsine(svel[i]) for i in range(3)])
    m4 = oracle.Oracle(64, 64, 64, lower, extent, nthreads=4)
    b = np.stack([m4.fftsine(svel[i]) for i in range(3)])
    assert np.abs(a - b).max() < 1.0e-15


def test_implicit_rk_known_answer():
    """unit-tests/test_implicit_rk.f90: with the source held at S = 1 and the
    damping D = 1, one integrating-factor RK4 step from q = 2 differs from the
    exact 2E + (1-E) (E = exp(-D dt)) by O(dt^5); the reference asserts
    < 1e-12 at dt = 0.0125.  The production stepper (impl_rk4.f90:76-207) is
    run with the source held fixed on the (kx, ky) = (1, 0) column, where the
    Hou-Li filter is 1 and the prefactor is chosen so that D = 1."""
    n = 16
    m = oracle.Oracle(n, n, n, [0, 0, 0], [1, 1, 1], hold_source=1)
    m.init_diffusion(1.0, 1.0)
    vhdis = m.table("vhdis")
    assert m.table("filt")[1, 0, 0] == 1.0
    dt = 0.1
    for _ in range(4):
        m.set("svor", np.full((3,) + m.shape, 2.0))
        m.set("svorts", np.full((3,) + m.shape, 1.0))
        m.ini_vor_mean = m.calc_vorticity_mean()
        m.set_diffusion(dt, 1.0 / vhdis[1, 0])
        m.step(0.0, dt)
        q = m.get("svor")[:, 1, 0, :]
        q0, exact = K.implicit_rk_reference(dt)
        scheme = K.if_rk4_constant(q0, 1.0, 1.0, dt)
        assert np.abs(q - scheme).max() < 1.0e-14
        err = abs(scheme - exact)
        dt *= 0.5
    assert err < 1.0e-12, err


def test_jacobi_eigenvalues_match_numpy():
    rng = np.random.default_rng(7)
    for _ in range(200):
        s = rng.standard_normal((3, 3))
        s = 0.5 * (s + s.T) * rng.uniform(0.01, 100)
        e = oracle.jacobi_eigenvalues(s)
        ref = np.sort(np.linalg.eigvalsh(s))[::-1]
        assert np.allclose(e, ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())


def test_transform_conventions():
    """stafft.f90:55-58: Hermitian storage, 1/sqrt(n); dst/dct self-inverse."""
    rng = np.random.default_rng(1)
    for n in (8, 32, 64, 128, 12, 30):
        x = rng.standard_normal(n)
        X = oracle.forfft(x)
        C = np.fft.fft(x) / np.sqrt(n)
        ref = np.zeros(n)
        ref[: n // 2 + 1] = C[: n // 2 + 1].real
        for k in range(1, (n - 1) // 2 + 1):
            ref[n - k] = C[k].imag
        assert np.abs(X - ref).max() < 1e-14
        assert np.abs(oracle.revfft(X) - x).max() < 1e-14
        y = rng.standard_normal(n)
        y[-1] = 0.0
        assert np.abs(oracle.dst(oracle.dst(y)) - y).max() < 1e-13
        z = rng.standard_normal(n + 1)
        assert np.abs(oracle.dct(oracle.dct(z)) - z).max() < 1e-13


def _beltrami_state(n):
    from ps3d_gb300 import ic
    lo, ex = ic.BELTRAMI_BOX["lower"], ic.BELTRAMI_BOX["extent"]
    o = oracle.Oracle(n, n, n, lo, ex)
    o.setup_fields(ic.beltrami_vorticity(n, n, n, lo, ex), None)
    o.vor2vel()
    return o, lo, ex


@pytest.mark.parametrize("n", [16, 32])
def test_pressure_of_beltrami_flow_is_bernoulli(n):
    """Derived pressure (fields_derived.f90:67-157): a Beltrami flow is a
    steady Euler solution with u x omega = 0, so grad p = -grad |u|^2/2 and
    p = -|u|^2/2 + const exactly."""
    o, _, _ = _beltrami_state(n)
    p = o.pressure()
    ke = 0.5 * np.sum(o.get("vel") ** 2, axis=0)
    a, b = p - p.mean(), -(ke - ke.mean())
    assert np.linalg.norm(a - b) / np.linalg.norm(b) < 1e-12


@pytest.mark.parametrize("n", [16, 32])
def test_horizontal_divergence_of_beltrami_flow(n):
    """Horizontal divergence (fields_derived.f90:161-182) against the analytic
    -dw/dz of the Beltrami field (k = l = 2, m = 1, u = omega / alpha):
    w = cos(mz) cos(kx + ly), so du/dx + dv/dy = m sin(mz) cos(kx + ly)."""
    o, lo, ex = _beltrami_state(n)
    d = o.horizontal_divergence()
    x = lo[0] + ex[0] / n * np.arange(n)
    y = lo[1] + ex[1] / n * np.arange(n)
    z = lo[2] + ex[2] / n * np.arange(n + 1)
    ref = np.sin(z)[None, None, :] * np.cos(2 * x[:, None] + 2 * y[None, :])[:, :, None]
    assert np.abs(d - ref).max() < 1e-12
