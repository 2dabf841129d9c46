"""GPU buoyancy path (the reference built with ENABLE_BUOYANCY) against the
oracle, through the C ABI.

FP64 form: tables, diffz and the set-up to 1e-12; sources, diagnostics and
steps to the same bars as the vorticity-only path (a near-Beltrami source is
a small difference of O(1) products, hence 1e-10 there).  Mixed form: FP32
transforms of the buoyancy with an FP64 state, within 1e-6 of the FP64
oracle over ten steps (relative L2 of the vorticity and of b')."""
import numpy as np
import pytest

import oracle
from ps3d_gb300 import Ps3dGpu, ic
from ps3d_gb300.solver import Ps3dError
from tests.parity_util import rel_l2

pytestmark = pytest.mark.gpu

BOX = ic.BELTRAMI_BOX


def _case(n, seed=3, bfsq=2.0, amp=2e-2):
    nx, ny, nz = n
    vor, pert = ic.beltrami_plus_perturbation(nx, ny, nz, seed=seed, amplitude=1e-3)
    btot = ic.stratified_buoyancy(nx, ny, nz, BOX["lower"], BOX["extent"], bfsq=bfsq, amplitude=amp,
                                  seed=seed + 1)
    return vor, pert, btot


def _pair(n, precision="fp64", **kw):
    kw.setdefault("buoyancy", True)
    kw.setdefault("cflmax", 0.5)
    o = oracle.Oracle(*n, BOX["lower"], BOX["extent"], **kw)
    g = Ps3dGpu(*n, BOX["lower"], BOX["extent"], precision=precision, **kw)
    vor, pert, btot = _case(n)
    teo, eno = o.setup_fields(vor, pert, buoy=btot)
    teg, eng = g.setup_fields(vor, pert, buoy=btot)
    return o, g, (teo, eno), (teg, eng)


@pytest.mark.parametrize("n", [(32, 32, 32), (16, 32, 64)], ids=lambda n: "x".join(map(str, n)))
def test_setup_tables_and_diffz(n):
    o, g, (teo, eno), (teg, eng) = _pair(n)
    assert abs(teg - teo) <= 1e-12 * teo and abs(eng - eno) <= 1e-12 * eno
    bo, vo = o.bfsq, o.bvisc
    bg, vg = g.buoyancy_params()
    assert abs(bg - bo) <= 1e-14 * bo and abs(vg - vo) <= 1e-12 * vo
    for name in ("dphim", "dphip", "bhdis", "bbarz"):
        np.testing.assert_allclose(g.table(name), o.table(name), rtol=1e-13, atol=1e-13)
    assert rel_l2(g.get("sbuoy"), o.get("sbuoy")) < 1e-13
    f = np.random.default_rng(1).standard_normal(g.shape)
    assert rel_l2(g.diffz(f), o.diffz(f)) < 1e-12


def test_source_adapt_and_diagnostics():
    o, g, _, _ = _pair((32, 32, 32))
    o.vor2vel()
    g.vor2vel()
    dto, do = o.adapt(0.0)
    dtg, dg = g.adapt(0.0)
    assert abs(dtg - dto) <= 1e-12 * dto
    for k in ("bfmax", "rmb", "bpref", "ggmax", "pref"):
        assert abs(dg[k] - do[k]) <= 1e-12 * max(abs(do[k]), 1e-300), (k, dg[k], do[k])
    dgo, dgg = o.buoyancy_diagnostics(), g.buoyancy_diagnostics()
    for a, b in zip(dgg, dgo):
        assert abs(a - b) <= 1e-12 * abs(b), (dgg, dgo)
    o.source()
    g.source()
    assert rel_l2(g.get("sbuoys"), o.get("sbuoys")) < 1e-11
    assert rel_l2(g.get("buoy"), o.get("buoy")) < 1e-13
    for c in range(3):
        assert rel_l2(g.get("svorts")[c], o.get("svorts")[c]) < 1e-10, c


def test_pressure_with_buoyancy():
    o, g, _, _ = _pair((32, 32, 32), f_cor=(0.0, 0.0, 0.7))
    o.vor2vel()
    g.vor2vel()
    po = o.pressure()
    pg, _ = g.derived_fields()
    assert rel_l2(pg, po) < 1e-12


@pytest.mark.parametrize("stepper", ["impl-diff-rk4", "cn2"])
def test_steps_match_oracle(stepper):
    o, g, _, _ = _pair((32, 32, 32), stepper=stepper, buoy_pretype="roll-mean-bfmax")
    t_o = t_g = 0.0
    for _ in range(5):
        t_o, do = o.advance(t_o)
        t_g, dg = g.advance(t_g)
        assert abs(dg["bfmax"] - do["bfmax"]) <= 1e-11 * do["bfmax"]
    assert abs(t_g - t_o) <= 1e-12 * t_o
    assert rel_l2(g.get("sbuoy"), o.get("sbuoy")) < 1e-12
    for c in range(3):
        assert rel_l2(g.get("svor")[c], o.get("svor")[c]) < 1e-12, c


def test_held_source_with_buoyancy():
    """hold_source keeps both sources fixed inside a step (the stepper alone)."""
    o, g, _, _ = _pair((16, 16, 16), hold_source=1)
    for m in (o, g):
        m.vor2vel()
        m.source()
    to = o.step(0.0, 0.01)
    tg = g.step(0.0, 0.01)
    assert tg == to
    assert rel_l2(g.get("sbuoy"), o.get("sbuoy")) < 1e-12


@pytest.mark.parametrize("stepper", ["impl-diff-rk4", "cn2"])
def test_mixed_tracks_fp64(stepper):
    n = (32, 32, 32)
    o, g, _, _ = _pair(n, precision="mixed", stepper=stepper)
    t_o = t_g = 0.0
    for _ in range(10):
        t_o, do = o.advance(t_o)
        t_g, dg = g.advance(t_g)
    assert abs(dg["bfmax"] - do["bfmax"]) <= 1e-5 * do["bfmax"]
    o.vor2vel()
    g.vor2vel()
    eb = rel_l2(g.get("sbuoy"), o.get("sbuoy"))
    ev = rel_l2(g.get("svor"), o.get("svor"))
    assert eb < 1e-6 and ev < 1e-6, (eb, ev)
    dgo, dgg = o.buoyancy_diagnostics(), g.buoyancy_diagnostics()
    assert abs(dgg[0] - dgo[0]) <= 1e-5 * dgo[0] and abs(dgg[1] - dgo[1]) <= 1e-5 * dgo[1]


def test_buoyancy_entry_points_refuse_cleanly():
    n = (16, 16, 16)
    g = Ps3dGpu(*n, BOX["lower"], BOX["extent"], buoyancy=True, precision="mixed")
    vor, pert, btot = _case(n)
    g.setup_fields(vor, pert, buoy=btot)
    host = np.ascontiguousarray(g.get("svor"))
    with pytest.raises(Ps3dError):
        g.advance_host(host, 0.0)
    with pytest.raises(Ps3dError):
        g.advance_graph(0.0, 1)
    plain = Ps3dGpu(*n, BOX["lower"], BOX["extent"])
    with pytest.raises(Ps3dError):
        plain.get("sbuoy")
    with pytest.raises(Ps3dError):
        plain.diffz(np.zeros(plain.shape))
    with pytest.raises(Ps3dError):
        plain.buoyancy_diagnostics()
    with pytest.raises(Ps3dError):
        Ps3dGpu(*n, BOX["lower"], BOX["extent"], pretype="roll-mean-bfmax")
