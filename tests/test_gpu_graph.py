"""Captured steps (CUDA graphs, adapt's scalar logic on the device) and the
batched driver, through the C ABI: same arithmetic as the host-driven
advance, so the states agree bitwise."""
import numpy as np
import pytest

from ps3d_gb300 import Ps3dGpu, batch_advance, ic

pytestmark = pytest.mark.gpu


def _model(n, seed, nz=None, prediss=30.0, amplitude=1e-3):
    nz = nz or n
    vor, pert = ic.beltrami_plus_perturbation(n, n, nz, seed=seed, amplitude=amplitude)
    m = Ps3dGpu(n, n, nz, ic.BELTRAMI_BOX["lower"], ic.BELTRAMI_BOX["extent"], precision="mixed",
                prediss=prediss, cflmax=0.5)
    m.setup_fields(vor, pert)
    return m


@pytest.mark.parametrize("n", [32, 64])
def test_graph_advance_matches_host_driven_advance(n):
    a, b = _model(n, 3), _model(n, 3)
    t_a = 0.0
    for _ in range(4):
        t_a, d_a = a.advance(t_a)
    t_b, d_b, ms = b.advance_graph(0.0, 4)
    assert t_a == t_b
    assert np.array_equal(a.get("svor"), b.get("svor"))
    for k in ("dt", "ke", "en", "hel", "ggmax", "vorch", "pref", "rmv"):
        assert d_a[k] == d_b[k], (k, d_a[k], d_b[k])
    assert ms > 0
    # continuing on the host after captured steps keeps the same trajectory
    t_a, _ = a.advance(t_a)
    t_b, _ = b.advance(t_b)
    assert np.array_equal(a.get("svor"), b.get("svor"))


def test_batch_of_uneven_runs_matches_individual_runs():
    """The batch step (every run's pieces on its own stream, one persistent
    launch per stage update over all runs' partner orbits, one CUDA graph per
    step) against the same runs advanced one by one: bitwise, over two
    calls (the second reuses the captured batch) and for a reordered subset
    (captured afresh)."""
    specs = [(32, 11, 10.0), (64, 12, 60.0), (128, 14, 30.0), (32, 13, 90.0)]
    batch = [_model(n, s, prediss=p) for n, s, p in specs]
    single = [_model(n, s, prediss=p) for n, s, p in specs]
    ts, ms = batch_advance(batch, [0.0] * len(batch), 2)
    ts, ms = batch_advance(batch, ts, 1)
    assert ms > 0
    for m, b, t in zip(single, batch, ts):
        tt = 0.0
        for _ in range(3):
            tt, _ = m.advance(tt)
        assert tt == t
        assert np.array_equal(m.get("svor"), b.get("svor"))
    sub = [batch[2], batch[0]]
    ts2, _ = batch_advance(sub, [ts[2], ts[0]], 1)
    for k, i in enumerate((2, 0)):
        tt, _ = single[i].advance(ts[i])
        assert tt == ts2[k]
        assert np.array_equal(single[i].get("svor"), batch[i].get("svor"))


def test_graph_refused_for_fp64_form():
    vor, pert = ic.beltrami_plus_perturbation(32, 32, 32, seed=1)
    m = Ps3dGpu(32, 32, 32, ic.BELTRAMI_BOX["lower"], ic.BELTRAMI_BOX["extent"], precision="fp64")
    m.setup_fields(vor, pert)
    with pytest.raises(Exception):
        m.advance_graph(0.0, 1)


@pytest.mark.parametrize("grid", [(512, 16, 8), (16, 512, 8), (256, 32, 40), (32, 128, 72)],
                         ids=lambda g: "x".join(map(str, g)))
def test_line_fft_shapes_all_match_oracle(grid):
    """Every kernel shape of the FP32 line FFTs (the autotuner's choices:
    512- and 256-thread blocks at 512 points, the TMA-fed persistent kernel
    at 128, 256 and 512 points) against the FP64 oracle, and the
    autotuner's record."""
    import oracle
    from tests.parity_util import rel_l2
    o = oracle.Oracle(*grid, [0.0, 0.0, 0.0], [1.0, 2.0, 0.5])
    g = Ps3dGpu(*grid, [0.0, 0.0, 0.0], [1.0, 2.0, 0.5], precision="mixed")
    shapes, ms = g.tuning()
    # shapes per line length (0 default, 1 256-thread blocks, 2 TMA-fed)
    have = {512: (0, 1, 2), 256: (0, 2), 128: (0, 2)}
    lengths = [grid[1], grid[0], grid[1], grid[0]]  # fwd y, fwd x, inv y, inv x
    for p in range(4):
        ws = have.get(lengths[p], ())
        if len(ws) > 1:
            assert shapes[p] in ws and all(ms[p][w] > 0 for w in ws), (p, shapes[p], ms[p])
    f = np.random.default_rng(5).standard_normal(o.shape)
    for w in (0, 1, 2):
        pin = [w if w in have.get(lengths[p], ()) else -1 for p in range(4)]
        g.set_tuning(pin)
        for op in ("fftxyp2s", "fftxys2p"):
            err = rel_l2(getattr(g, op)(f), getattr(o, op)(f))
            assert err < 2e-6, (w, op, err)
