"""CPU checks of the closure's host logic.

The spectral cut that turns a fine mixed-spectral field into the coarse
grid's representation (closure.spectral_cut) is checked against the oracle's
field_decompose_physical (inversion_utils.f90:549-557) run on both grids:
for a field whose modes the coarse grid resolves, cutting the fine
decomposition must give the coarse decomposition.
"""
import numpy as np
import pytest

import oracle
from ps3d_gb300 import closure, ic

LO, EX = ic.BELTRAMI_BOX["lower"], ic.BELTRAMI_BOX["extent"]


def band_limited(nx, ny, nz):
    """Interior sine modes 3 and 5 in z, horizontal modes up to 3, and a
    harmonic (sinh) profile carrying non-zero wall values."""
    x = LO[0] + EX[0] / nx * np.arange(nx)
    y = LO[1] + EX[1] / ny * np.arange(ny)
    z = LO[2] + EX[2] / nz * np.arange(nz + 1)
    X, Y, Zz = np.meshgrid(x, y, z, indexing="ij")
    s = Zz - LO[2]
    f = np.cos(2 * X) * np.cos(Y) * np.sin(3 * s)
    f += 0.5 * np.sin(X + 0.3) * np.cos(3 * Y) * np.sin(5 * s)
    f += 0.25 * np.cos(X) * np.sinh(s) / np.sinh(EX[2])
    f += 0.1 * np.sin(2 * Y) * np.sinh(2 * (EX[2] - s)) / np.sinh(2 * EX[2])
    return f


@pytest.mark.parametrize("fine,coarse", [((32, 32, 32), (16, 16, 16)), ((32, 16, 64), (16, 8, 16)),
                                         ((64, 64, 32), (16, 32, 16))])
def test_cut_matches_coarse_decomposition(fine, coarse):
    of = oracle.Oracle(*fine, LO, EX)
    oc = oracle.Oracle(*coarse, LO, EX)
    sf = of.decompose_physical(band_limited(*fine))
    sc = oc.decompose_physical(band_limited(*coarse))
    cut = closure.spectral_cut(sf, *coarse)
    err = np.linalg.norm(cut - sc) / np.linalg.norm(sc)
    assert err < 1e-12, err
    # and back to the physical coarse grid
    back = oc.combine_physical(cut)
    assert np.allclose(back, band_limited(*coarse), atol=1e-12)


def test_cut_drops_unresolved_modes():
    fine, coarse = (32, 32, 32), (16, 16, 16)
    of = oracle.Oracle(*fine, LO, EX)
    x = LO[0] + EX[0] / 32 * np.arange(32)
    z = LO[2] + EX[2] / 32 * np.arange(33)
    f = np.cos(9 * x)[:, None, None] * np.ones(32)[None, :, None] * np.sin(3 * (z - LO[2]))[None, None, :]
    g = np.ones(32)[:, None, None] * np.ones(32)[None, :, None] * np.sin(20 * (z - LO[2]))[None, None, :]
    cut = closure.spectral_cut(of.decompose_physical(f + g), *coarse)
    assert np.max(np.abs(cut)) < 1e-12


def test_cut_is_identity_on_the_same_grid_except_nyquist():
    rng = np.random.default_rng(0)
    a = rng.standard_normal((3, 16, 8, 17))
    b = closure.spectral_cut(a, 16, 8, 16)
    a[:, 8, :, :] = 0.0
    a[:, :, 4, :] = 0.0
    assert np.array_equal(a, b)


def test_parameter_layout():
    p = np.arange(closure.NPARAM, dtype=np.float32)
    views = closure.param_views(p)
    assert [w.shape for w, _ in views] == [(27, 6, 32), (27, 32, 32), (27, 32, 32), (27, 32, 3)]
    assert views[-1][1][-1] == closure.NPARAM - 1


def test_spectrum_interpolation_and_shell_error():
    from ps3d_gb300 import closure_case as cc
    k = np.arange(30, dtype=float)
    series = [(0.0, 1.0 + k), (0.5, 3.0 + k), (1.5, 5.0 + k)]
    assert np.allclose(cc.at_time(series, 0.25), 2.0 + k)
    assert np.allclose(cc.at_time(series, 1.0), 4.0 + k)
    assert np.allclose(cc.at_time(series, -1.0), 1.0 + k)   # before the first sample
    assert np.allclose(cc.at_time(series, 9.0), 5.0 + k)    # after the last
    truth = 1.0 + k
    model = truth.copy()
    model[3] *= 1.5
    model[21] *= 0.9
    model[25] *= 10.0                                        # beyond shell 21: ignored
    mx, mean = closure.shell_error(model, truth, kmax=21)
    assert abs(mx - 0.5) < 1e-12 and abs(mean - 0.6 / 21) < 1e-12


def test_variant_parsing():
    from ps3d_gb300 import closure_case as cc
    v = cc.parse_variants("plain=30,net=10:net+every+g0.5,m=0:net+mma")
    assert v == [("plain", 30.0, set()), ("net", 10.0, {"net", "every", "g0.5"}), ("m", 0.0, {"net", "mma"})]
    assert [x[0] for x in cc.parse_variants(cc.DEFAULT_VARIANTS)][0] == "plain"
