"""GPU library vs CPU oracle on identical FP64 inputs (the parity gate).

Every call goes through the C ABI (libps3d_gpu.so via ctypes).  Tolerances:
relative L2 1e-12 per field per step and 1e-10 on the energy / enstrophy /
helicity series for the plain FP64 form (the bar of the path), transform-level
operators 1e-13.
"""
import numpy as np
import pytest

import oracle
from ps3d_gb300 import Ps3dGpu
from tests import kat_cases as K
from tests.parity_util import beltrami_case, rel_l2
from ps3d_gb300 import ic

pytestmark = pytest.mark.gpu

FIELD_TOL = 1.0e-12
SERIES_TOL = 1.0e-10
OP_TOL = 1.0e-13

GRIDS = [
    (32, 32, 32, [0.0, 0.0, -0.5 * np.pi], [2 * np.pi, 2 * np.pi, np.pi]),
    (16, 32, 64, [-0.5, -0.5, 0.0], [1.0, 2.0, 1.5]),
    (64, 16, 8, [0.0, -1.0, 0.0], [3.0, 2.0, 0.5]),
]


def _pair(nx, ny, nz, lo, ex, **kw):
    return (oracle.Oracle(nx, ny, nz, lo, ex, **kw),
            Ps3dGpu(nx, ny, nz, lo, ex, **kw))


@pytest.mark.parametrize("grid", GRIDS, ids=lambda g: "x".join(map(str, g[:3])))
@pytest.mark.parametrize("op", ["fftxyp2s", "fftxys2p", "diffx", "diffy", "fftsine", "fftcosine",
                                "central_diffz", "decompose_semi_spectral",
                                "combine_semi_spectral", "decompose_physical", "combine_physical"])
def test_field_operators_match_oracle(grid, op):
    o, g = _pair(*grid)
    f = np.random.default_rng(3).standard_normal(o.shape)
    a = getattr(g, op)(f)
    b = getattr(o, op)(f)
    assert rel_l2(a, b) < OP_TOL, (op, rel_l2(a, b))


@pytest.mark.parametrize("grid", GRIDS[:2], ids=lambda g: "x".join(map(str, g[:3])))
@pytest.mark.parametrize("name", ["k2l2", "k2l2i", "filt", "green", "phim", "phip", "thetam", "thetap",
                                  "dthetam", "dthetap", "gamtop", "gambot", "rkx", "rky", "rkz"])
def test_tables_match_oracle(grid, name):
    o, g = _pair(*grid)
    assert rel_l2(g.table(name), o.table(name)) < OP_TOL


def test_roundtrips_and_empty_input():
    o, g = _pair(*GRIDS[0])
    f = np.random.default_rng(5).standard_normal(o.shape)
    assert rel_l2(g.fftxys2p(g.fftxyp2s(f)), f) < OP_TOL
    assert rel_l2(g.combine_physical(g.decompose_physical(f)), f) < OP_TOL
    z = np.zeros(o.shape)
    for op in ("fftxyp2s", "decompose_physical", "fftcosine"):
        assert np.all(getattr(g, op)(z) == 0.0)


@pytest.mark.parametrize("name", sorted(K.VOR2VEL_CASES))
def test_vor2vel_known_answer_on_gpu(name):
    """The reference's unit-tests/test_vor2vel_{1..5}.f90 through the GPU."""
    c = K.VOR2VEL_CASES[name]()
    g = Ps3dGpu(c["nx"], c["ny"], c["nz"], c["lower"], c["extent"])
    svor = np.stack([g.decompose_physical(c["vor"][i]) for i in range(3)])
    g.set("svor", svor)
    g.vor2vel()
    err = np.abs(g.get("vel") - c["vel"]).max()
    assert err < c["atol"], (name, err)


@pytest.mark.parametrize("name", ["diffz_1", "diffz_2", "diffz_3", "diffz_4"])
def test_diffz_known_answer_on_gpu(name):
    c = K.diffz_cases()[name]
    g = Ps3dGpu(c["nx"], c["ny"], c["nz"], c["lower"], c["extent"])
    assert np.abs(g.central_diffz(c["f"]) - c["dfdz"]).max() < c["atol"]


@pytest.mark.parametrize("name", ["diffx", "diffy"])
def test_diffxy_known_answer_on_gpu(name):
    c = K.diffxy_cases()[name]
    g = Ps3dGpu(c["nx"], c["ny"], c["nz"], c["lower"], c["extent"])
    fs = g.fftxyp2s(c["f"])
    ds = g.diffx(fs) if c["axis"] == "x" else g.diffy(fs)
    assert np.abs(g.fftxys2p(ds) - c["df"]).max() < c["atol"]


def test_implicit_rk_known_answer_on_gpu():
    """unit-tests/test_implicit_rk.f90 through the GPU stepper (see the oracle
    port in test_oracle_kat.py)."""
    n = 16
    g = Ps3dGpu(n, n, n, [0, 0, 0], [1, 1, 1], hold_source=1)
    g.init_diffusion(1.0, 1.0)
    vhdis = g.table("vhdis")
    dt = 0.1
    for _ in range(4):
        g.set("svor", np.full((3,) + g.shape, 2.0))
        g.set("svorts", np.full((3,) + g.shape, 1.0))
        g.ini_vor_mean = g.calc_vorticity_mean()
        g.set_diffusion(dt, 1.0 / vhdis[1, 0])
        g.step(0.0, dt)
        q = g.get("svor")[:, 1, 0, :]
        q0, exact = K.implicit_rk_reference(dt)
        assert np.abs(q - K.if_rk4_constant(q0, 1.0, 1.0, dt)).max() < 1.0e-14
        dt *= 0.5


def _setup_both(n, stepper="impl-diff-rk4", seed=1, cflmax=0.5, **kw):
    lo, ex, vor, pert = beltrami_case(n, seed=seed)
    o = oracle.Oracle(n, n, n, lo, ex, stepper=stepper, cflmax=cflmax, **kw)
    g = Ps3dGpu(n, n, n, lo, ex, stepper=stepper, cflmax=cflmax, **kw)
    te_o, en_o = o.setup_fields(vor, pert)
    te_g, en_g = g.setup_fields(vor, pert)
    assert abs(te_g - te_o) <= SERIES_TOL * abs(te_o)
    assert abs(en_g - en_o) <= SERIES_TOL * abs(en_o)
    return o, g


def test_setup_vor2vel_source_adapt_match_oracle():
    o, g = _setup_both(32)
    np.testing.assert_allclose(g.ini_vor_mean, o.ini_vor_mean, rtol=0, atol=1e-14)
    for f in ("svor", "vor", "vel", "svel"):
        for c in range(3):
            assert rel_l2(g.get(f)[c], o.get(f)[c]) < FIELD_TOL, (f, c)
    g.source()
    o.source()
    # The tendency of a near-Beltrami flow (u parallel to omega) is a small
    # difference of O(1) products: u x omega cancels to the 1e-3 level of the
    # perturbation, so FP64 rounding shows up ~1e3 times larger relative to
    # the tendency than to the state.  The state after a step is checked at
    # the 1e-12 bar below.
    for c in range(3):
        assert rel_l2(g.get("svorts")[c], o.get("svorts")[c]) < 1.0e-10, c
    dtg, dg = g.adapt(0.0)
    dto, do = o.adapt(0.0)
    assert abs(dtg - dto) <= 1e-12 * dto
    for k in ("ke", "en", "hel", "vortmax", "vortrms", "vorch", "ggmax", "usggmax", "lsggmax",
              "umax", "vmax", "wmax", "rmv", "pref"):
        assert abs(dg[k] - do[k]) <= 1e-11 * max(abs(do[k]), 1e-300), (k, dg[k], do[k])
    np.testing.assert_allclose(g.table("vhdis"), o.table("vhdis"), rtol=1e-13, atol=0)


@pytest.mark.parametrize("stepper", ["impl-diff-rk4", "cn2"])
def test_one_step_matches_oracle(stepper):
    o, g = _setup_both(32, stepper=stepper)
    tg, dg = g.advance(0.0)
    to, do = o.advance(0.0)
    assert abs(tg - to) <= 1e-13 * to
    for c in range(3):
        assert rel_l2(g.get("svor")[c], o.get("svor")[c]) < FIELD_TOL


def test_multi_step_parity_per_step():
    """Per-step relative L2 of each vorticity component and the energy /
    enstrophy / helicity series over 200 steps at 32^3 against the oracle,
    measured against a shadow oracle run that carries the GPU's own per-step
    rounding differences (tests.parity_util.multi_step_parity); the worst
    ratio of GPU error to shadow is printed.  (128^3 over 200 steps:
    test_gpu_parity_config2.py.)"""
    from tests.parity_util import multi_step_parity
    ratio, at, series, eps = multi_step_parity(32, 200, check_every=10)
    print(f"32^3 x 200 steps: worst local (one-step) error {eps:.3g}; worst GPU/shadow ratio {ratio:.3g} at "
          f"(step, comp, err, floor) {at}; worst series error {series:.3g}")


def test_mixed_precision_tracks_fp64():
    """Mixed form (FP32 transforms/products/stages, FP64 state, inversion
    and reductions) against the FP64 oracle after 20 steps at 32^3."""
    lo, ex, vor, pert = beltrami_case(32, seed=2)
    o = oracle.Oracle(32, 32, 32, lo, ex, cflmax=0.5)
    g = Ps3dGpu(32, 32, 32, lo, ex, cflmax=0.5, precision="mixed")
    o.setup_fields(vor, pert)
    g.setup_fields(vor, pert)
    t_o = t_g = 0.0
    for _ in range(20):
        t_g, dg = g.advance(t_g)
        t_o, do = o.advance(t_o)
    # compare solenoidal states: the reference projects svor at the start of
    # the next vor2vel; the mixed form keeps it projected
    o.vor2vel()
    g.vor2vel()
    err = rel_l2(g.get("svor"), o.get("svor"))
    assert err < 1.0e-6, err
    assert abs(dg["ke"] - do["ke"]) < 1e-6 * do["ke"]


def test_advance_host_equals_resident_advance():
    lo, ex, vor, pert = beltrami_case(32, seed=4)
    a = Ps3dGpu(32, 32, 32, lo, ex)
    b = Ps3dGpu(32, 32, 32, lo, ex)
    a.setup_fields(vor, pert)
    b.setup_fields(vor, pert)
    host = np.ascontiguousarray(b.get("svor"))
    t_a = t_b = 0.0
    for _ in range(3):
        t_a, _ = a.advance(t_a)
        t_b, _ = b.advance_host(host, t_b)
    assert np.array_equal(a.get("svor"), host)
    assert t_a == t_b


MIXED_OP_TOL = 2.0e-6


@pytest.mark.parametrize("nz", [16, 32, 64, 128, 256, 512])
@pytest.mark.parametrize("op", ["fftsine", "fftcosine", "decompose_semi_spectral", "combine_semi_spectral",
                                "fftxyp2s", "fftxys2p", "decompose_physical", "combine_physical",
                                "central_diffz", "diffx", "diffy"])
def test_mixed_field_operators_match_oracle(nz, op):
    """FP32 operators of the mixed form (warp-per-column-pair z transforms
    for nz = 32..512, shared-memory Stockham otherwise) against the FP64
    oracle, relative L2 within 2e-6."""
    grid = (16, 8, nz, [0.0, 0.0, -0.5], [2 * np.pi, 1.0, 1.0])
    o = oracle.Oracle(*grid)
    g = Ps3dGpu(*grid, precision="mixed")
    f = np.random.default_rng(11).standard_normal(o.shape)
    err = rel_l2(getattr(g, op)(f), getattr(o, op)(f))
    assert err < MIXED_OP_TOL, (op, nz, err)


MIXED_GRIDS = [(32, 32, 64), (16, 16, 128), (16, 8, 256), (8, 8, 512)]


@pytest.mark.parametrize("grid", MIXED_GRIDS, ids=lambda g: "x".join(map(str, g)))
def test_mixed_vor2vel_and_source_match_oracle(grid):
    """Mixed-form vor2vel (fused vertical-velocity column kernel) and
    source (the tendency's decompositions, the third fused with the z part
    of its solenoidal projection) against the FP64 oracle on the same state:
    velocity and vorticity within 2e-6, the tendency within 2e-4.  The
    tendency of a near-Beltrami flow is a difference of nearly equal
    products: rounding vel and vor alone to FP32 moves the oracle's tendency
    by about 1e-5 (relative L2) at these sizes.  Like the reference's source,
    the mixed source leaves the tendency unprojected; the projection happens
    in the stage update."""
    nx, ny, nz = grid
    lo, ex = ic.BELTRAMI_BOX["lower"], ic.BELTRAMI_BOX["extent"]
    vor, pert = ic.beltrami_plus_perturbation(nx, ny, nz, seed=5, amplitude=1.0e-2)
    o = oracle.Oracle(nx, ny, nz, lo, ex)
    g = Ps3dGpu(nx, ny, nz, lo, ex, precision="mixed")
    o.setup_fields(vor, pert)
    g.setup_fields(vor, pert)
    o.vor2vel()
    g.vor2vel()
    # FP32 transform error grows with the column length: 2e-6 up to nz = 256,
    # 1e-5 at nz = 512 (the vorticity, through the plain combine, shows the
    # same growth as the velocity)
    tol = MIXED_OP_TOL if nz <= 256 else 1.0e-5
    for name in ("vel", "vor", "svel"):
        err = rel_l2(g.get(name), o.get(name))
        assert err < tol, (name, err)
    o.source()
    g.source()
    err = rel_l2(g.get("svorts"), o.get("svorts"))
    assert err < 2.0e-4, err


PRODUCT_LINE_GRIDS = [(64, 64, 64), (16, 128, 64), (16, 256, 40), (8, 512, 64), (8, 1024, 64), (8, 512, 120)]


def _mixed_source(grid, fuse, monkeypatch):
    """svorts of the mixed source on the seeded perturbed Beltrami state,
    with the products formed inside the forward y-line kernel (fuse "1") or
    by the separate products kernel ("0"); the choice is read when the
    context is created."""
    nx, ny, nz = grid
    lo, ex = ic.BELTRAMI_BOX["lower"], ic.BELTRAMI_BOX["extent"]
    vor, pert = ic.beltrami_plus_perturbation(nx, ny, nz, seed=6, amplitude=1.0e-2)
    monkeypatch.setenv("PS3D_FUSE_PRODUCTS", fuse)
    g = Ps3dGpu(nx, ny, nz, lo, ex, precision="mixed")
    monkeypatch.delenv("PS3D_FUSE_PRODUCTS")
    g.setup_fields(vor, pert)
    g.vor2vel()
    g.source()
    return g.get("svorts"), vor, pert


@pytest.mark.parametrize("grid", PRODUCT_LINE_GRIDS, ids=lambda g: "x".join(map(str, g)))
def test_mixed_source_fused_products_match_oracle(grid, monkeypatch):
    """For y line lengths 64..1024 the mixed source can form the five
    products (and the z derivatives of two of them) inside the forward
    y-line kernel (the default for fields of 2^24 elements and more; forced
    here) and the tendency components inside the column kernels that
    decompose them.  (1) The fused products give bitwise the tendency of the
    separate products kernel with the plain line transforms.  (2) Against
    the FP64 oracle on the same state: the tendency of a near-Beltrami flow
    is a small difference of nearly equal products, so the FP32 rounding of
    the products and of the line transforms shows at the 1e-4 level, growing
    with the line length: measured on a GB300, 5.8e-5 (64^3), 1.5e-4
    (ny = 256), 2.5e-4 (ny = 512), 5.4e-4 (ny = 1024), spread evenly over the
    levels; the tolerance is about 1.5x that.  The column counts put
    z-derivatives across the edges of the kernel's 32-level z tiles
    (nz = 64, 120) and the top wall inside a tile (nz = 40, 120; those
    column lengths take the unfused tendency assembly)."""
    nx, ny, nz = grid
    fused, vor, pert = _mixed_source(grid, "1", monkeypatch)
    plain, _, _ = _mixed_source(grid, "0", monkeypatch)
    assert np.array_equal(fused, plain)
    lo, ex = ic.BELTRAMI_BOX["lower"], ic.BELTRAMI_BOX["extent"]
    o = oracle.Oracle(nx, ny, nz, lo, ex)
    o.setup_fields(vor, pert)
    o.vor2vel()
    o.source()
    tol = {64: 1.0e-4, 128: 2.0e-4, 256: 2.5e-4, 512: 4.0e-4, 1024: 8.0e-4}[max(nx, ny)]
    err = rel_l2(fused, o.get("svorts"))
    assert err < tol, err


@pytest.mark.parametrize("n", [64])
def test_mixed_steps_track_fp64_at_fused_sizes(n):
    """Ten mixed steps at 64^3 (fused column kernels active) against the FP64
    oracle: solenoidal state within 1e-6."""
    lo, ex, vor, pert = beltrami_case(n, seed=6)
    o = oracle.Oracle(n, n, n, lo, ex, cflmax=0.5)
    g = Ps3dGpu(n, n, n, lo, ex, cflmax=0.5, precision="mixed")
    o.setup_fields(vor, pert)
    g.setup_fields(vor, pert)
    t_o = t_g = 0.0
    for _ in range(10):
        t_g, dg = g.advance(t_g)
        t_o, do = o.advance(t_o)
    o.vor2vel()
    g.vor2vel()
    err = rel_l2(g.get("svor"), o.get("svor"))
    assert err < 1.0e-6, err
    assert abs(dg["ke"] - do["ke"]) < 1e-6 * do["ke"]


@pytest.mark.parametrize("grid", [(64, 128, 8), (256, 64, 8), (512, 16, 8), (16, 512, 8), (1024, 8, 8),
                                  (8, 1024, 8)], ids=lambda g: "x".join(map(str, g)))
@pytest.mark.parametrize("op", ["fftxyp2s", "fftxys2p", "decompose_physical", "combine_physical"])
def test_mixed_line_transforms_match_oracle(grid, op):
    """FP32 register-butterfly line FFTs of the mixed form (x and y lines of
    64..1024 points; the inverse reads the Hermitian rows in its first
    pass) against the FP64 oracle, relative L2 within 2e-6."""
    o = oracle.Oracle(*grid, [0.0, 0.0, 0.0], [1.0, 2.0, 0.5])
    g = Ps3dGpu(*grid, [0.0, 0.0, 0.0], [1.0, 2.0, 0.5], precision="mixed")
    f = np.random.default_rng(12).standard_normal(o.shape)
    err = rel_l2(getattr(g, op)(f), getattr(o, op)(f))
    assert err < MIXED_OP_TOL, (op, grid, err)


@pytest.mark.parametrize("grid", [(32, 32, 32), (64, 32, 64)], ids=lambda g: "x".join(map(str, g)))
def test_mixed_adapt_diagnostics_match_oracle(grid):
    """Mixed-form adapt (FP32 strain eigenvalues in closed form, FP32
    compensated sums) against the FP64 oracle's Jacobi eigenvalues: the time
    step and every diagnostic within 2e-5 relative (the FP32 gradients carry
    about 1e-6 relative rounding)."""
    nx, ny, nz = grid
    lo, ex = ic.BELTRAMI_BOX["lower"], ic.BELTRAMI_BOX["extent"]
    vor, pert = ic.beltrami_plus_perturbation(nx, ny, nz, seed=8, amplitude=5.0e-2)
    o = oracle.Oracle(nx, ny, nz, lo, ex, pretype="vorch")
    g = Ps3dGpu(nx, ny, nz, lo, ex, pretype="vorch", precision="mixed")
    o.setup_fields(vor, pert)
    g.setup_fields(vor, pert)
    dtg, dg = g.adapt(0.0)
    dto, do = o.adapt(0.0)
    assert abs(dtg - dto) <= 2e-5 * dto, (dtg, dto)
    for k in ("ke", "en", "hel", "vortmax", "vortrms", "vorch", "ggmax", "usggmax", "lsggmax",
              "umax", "vmax", "wmax", "pref"):
        assert abs(dg[k] - do[k]) <= 2e-5 * max(abs(do[k]), 1e-300), (k, dg[k], do[k])


def test_mixed_advance_host_matches_resident_and_projects_changes():
    """advance_host in the mixed form: an unchanged host state continues the
    resident trajectory bitwise; a changed one is projected first, exactly as
    set_field does."""
    lo, ex, vor, pert = beltrami_case(64, seed=9)
    a = Ps3dGpu(64, 64, 64, lo, ex, precision="mixed")
    b = Ps3dGpu(64, 64, 64, lo, ex, precision="mixed")
    a.setup_fields(vor, pert)
    b.setup_fields(vor, pert)
    host = np.ascontiguousarray(b.get("svor"))
    t_a = t_b = 0.0
    for _ in range(3):
        t_a, _ = a.advance(t_a)
        t_b, _ = b.advance_host(host, t_b)
    assert np.array_equal(a.get("svor"), host)
    assert t_a == t_b
    # a host-side change (not solenoidal) goes through the FP64 projection
    kick = 1e-3 * np.random.default_rng(1).standard_normal(host.shape)
    changed = host + kick
    a.set("svor", changed)
    t_a, _ = a.advance(t_a)
    host[...] = changed
    t_b, _ = b.advance_host(host, t_b)
    assert np.array_equal(a.get("svor"), host)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_advance_host_page_locked_equals_pageable(precision):
    """A state buffer from ps3d_gpu_host_alloc is read and written in place by
    the device (zero copy; in the mixed form the read and its comparison run
    beside the first right-hand side); a plain numpy buffer goes through the
    staging copies.  Both give the same state bitwise, including a host-side
    change (which makes the mixed form evaluate the first right-hand side
    again)."""
    from ps3d_gb300.solver import PinnedArray
    lo, ex, vor, pert = beltrami_case(32, seed=12)
    a = Ps3dGpu(32, 32, 32, lo, ex, precision=precision)
    b = Ps3dGpu(32, 32, 32, lo, ex, precision=precision)
    a.setup_fields(vor, pert)
    b.setup_fields(vor, pert)
    plain = np.ascontiguousarray(a.get("svor"))
    locked = PinnedArray(plain.shape)
    try:
        locked.array[...] = plain
        t_a = t_b = 0.0
        for i in range(3):
            if i == 2:
                kick = 1e-3 * np.random.default_rng(2).standard_normal(plain.shape)
                plain += kick
                locked.array[...] += kick
            t_a, da = a.advance_host(plain, t_a)
            t_b, db = b.advance_host(locked.array, t_b)
            assert np.array_equal(plain, locked.array)
            # rmv: adapt's rolling mean, which a changed state's second
            # evaluation of the first right-hand side must not advance twice
            assert t_a == t_b and da["ke"] == db["ke"] and da["rmv"] == db["rmv"]
    finally:
        locked.close()


@pytest.mark.parametrize("grid", [(32, 32, 32), (16, 32, 64), (40, 30, 24)], ids=lambda g: "x".join(map(str, g)))
def test_advance_host_page_locked_unaligned_equals_aligned(grid):
    """Page-locked state buffers are moved over the host link as 16-byte
    pairs when 16-byte aligned, and column by column otherwise; a buffer
    starting 8 bytes into a page-locked allocation takes the second route.
    Both give the state bitwise, and both see a host-side change."""
    from ps3d_gb300.solver import PinnedArray
    nx, ny, nz = grid
    lo, ex = ic.BELTRAMI_BOX["lower"], ic.BELTRAMI_BOX["extent"]
    vor, pert = ic.beltrami_plus_perturbation(nx, ny, nz, seed=13)
    a = Ps3dGpu(nx, ny, nz, lo, ex, precision="mixed")
    b = Ps3dGpu(nx, ny, nz, lo, ex, precision="mixed")
    a.setup_fields(vor, pert)
    b.setup_fields(vor, pert)
    state = np.ascontiguousarray(a.get("svor"))
    al = PinnedArray(state.shape)
    raw = PinnedArray((state.size + 1,))
    try:
        un = raw.array[1:].reshape(state.shape)
        assert un.ctypes.data % 16 == 8 and al.array.ctypes.data % 16 == 0
        al.array[...] = state
        un[...] = state
        t_a = t_b = 0.0
        for i in range(3):
            if i == 1:
                kick = 1e-3 * np.random.default_rng(3).standard_normal(state.shape)
                al.array[...] += kick
                un[...] += kick
            t_a, da = a.advance_host(al.array, t_a)
            t_b, db = b.advance_host(un, t_b)
            assert np.array_equal(al.array, un)
            assert t_a == t_b and da["ke"] == db["ke"] and da["rmv"] == db["rmv"]
        assert np.array_equal(a.get("svor"), al.array)
    finally:
        al.close()
        raw.close()


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("mixed", 1e-4)])
@pytest.mark.parametrize("grid", [(32, 32, 32), (16, 32, 64)], ids=lambda g: "x".join(map(str, g)))
def test_derived_pressure_and_divergence_match_oracle(grid, precision, tol):
    """Pressure and horizontal divergence (fields_derived.f90:67-182) of a
    perturbed Beltrami state against the oracle: 1e-12 in FP64, 1e-4 in the
    mixed form (FP32 products of the velocity gradients)."""
    nx, ny, nz = grid
    lo, ex = ic.BELTRAMI_BOX["lower"], ic.BELTRAMI_BOX["extent"]
    vor, pert = ic.beltrami_plus_perturbation(nx, ny, nz, seed=4, amplitude=1e-2)
    o = oracle.Oracle(nx, ny, nz, lo, ex)
    g = Ps3dGpu(nx, ny, nz, lo, ex, precision=precision)
    o.setup_fields(vor, pert)
    g.setup_fields(vor, pert)
    o.vor2vel()
    g.vor2vel()
    p, dl = g.derived_fields()
    assert rel_l2(p, o.pressure()) < tol
    assert rel_l2(dl, o.horizontal_divergence()) < tol


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("mixed", 1e-5)])
@pytest.mark.parametrize("grid", [(32, 32, 32), (16, 32, 64)], ids=lambda g: "x".join(map(str, g)))
def test_ke_spectrum_matches_oracle(grid, precision, tol):
    """Kinetic-energy shell spectrum (genspec.f90:42-123) against the oracle:
    same shells and dk, every shell within tol of the largest, sum(spec) dk
    equal to the domain-average kinetic energy."""
    nx, ny, nz = grid
    lo, ex = ic.BELTRAMI_BOX["lower"], ic.BELTRAMI_BOX["extent"]
    vor, pert = ic.beltrami_plus_perturbation(nx, ny, nz, seed=6, amplitude=1e-2)
    o = oracle.Oracle(nx, ny, nz, lo, ex)
    g = Ps3dGpu(nx, ny, nz, lo, ex, precision=precision)
    o.setup_fields(vor, pert)
    g.setup_fields(vor, pert)
    o.vor2vel()
    g.vor2vel()
    so, dko = o.ke_spectrum()
    sg, dkg = g.ke_spectrum()
    assert len(sg) == len(so) and dkg == dko
    assert np.abs(sg - so).max() <= tol * so.max()
    ke = o.energy_series()[0]
    assert abs(sg.sum() * dkg - ke) <= 1e-6 * ke


@pytest.mark.parametrize("grid,stepper", [((64, 64, 64), "cn2"), ((32, 32, 32), "cn2"),
                                          ((64, 32, 128), "impl-diff-rk4")],
                         ids=["cn2-64", "cn2-32", "rk4-64x32x128"])
def test_mixed_steps_other_steppers_and_shapes(grid, stepper):
    """Mixed form over ten steps against the FP64 oracle for the cn2 stepper
    and a non-cubic grid: solenoidal state within 1e-6."""
    nx, ny, nz = grid
    lo, ex = ic.BELTRAMI_BOX["lower"], ic.BELTRAMI_BOX["extent"]
    vor, pert = ic.beltrami_plus_perturbation(nx, ny, nz, seed=10)
    o = oracle.Oracle(nx, ny, nz, lo, ex, cflmax=0.5, stepper=stepper)
    g = Ps3dGpu(nx, ny, nz, lo, ex, cflmax=0.5, stepper=stepper, precision="mixed")
    o.setup_fields(vor, pert)
    g.setup_fields(vor, pert)
    t_o = t_g = 0.0
    for _ in range(10):
        t_g, dg = g.advance(t_g)
        t_o, do = o.advance(t_o)
    o.vor2vel()
    g.vor2vel()
    err = rel_l2(g.get("svor"), o.get("svor"))
    assert err < 1.0e-6, err
    assert abs(t_g - t_o) <= 1e-6 * t_o


@pytest.mark.parametrize("n", [32, 64])
def test_mixed_held_source_step_matches_oracle(n):
    """hold_source in the mixed form: the source of the first right-hand side
    (with the z part of its projection) is held over the four substeps; the
    stepped state against the oracle's within 1e-6 (32^3: the
    shared-memory column transforms, 64^3: the warp column kernels)."""
    lo, ex, vor, pert = beltrami_case(n, seed=13, amplitude=1e-2)
    o = oracle.Oracle(n, n, n, lo, ex, hold_source=1)
    g = Ps3dGpu(n, n, n, lo, ex, hold_source=1, precision="mixed")
    o.setup_fields(vor, pert)
    g.setup_fields(vor, pert)
    for m in (o, g):
        m.vor2vel()
        m.source()
        dt, _ = m.adapt(0.0)
        m.step(0.0, dt)
        m.vor2vel()
    err = rel_l2(g.get("svor"), o.get("svor"))
    assert err < 1.0e-6, err


@pytest.mark.parametrize("grid", [(64, 64, 64), (128, 128, 40), (256, 256, 8), (512, 512, 72), (1024, 1024, 8)],
                         ids=lambda g: "x".join(map(str, g)))
@pytest.mark.parametrize("op", ["fftxyp2s", "fftxys2p", "decompose_physical", "combine_physical"])
def test_mixed_square_plane_transforms_match_oracle(grid, op):
    """FP32 horizontal transforms of square planes (the benchmark's shape)
    at every line length of the register-butterfly kernels, over one to
    three tiles of 32 levels, against the FP64 oracle within 2e-6."""
    o = oracle.Oracle(*grid, [0.0, 0.0, 0.0], [2.0, 2.0, 0.5])
    g = Ps3dGpu(*grid, [0.0, 0.0, 0.0], [2.0, 2.0, 0.5], precision="mixed")
    f = np.random.default_rng(14).standard_normal(o.shape)
    err = rel_l2(getattr(g, op)(f), getattr(o, op)(f))
    assert err < MIXED_OP_TOL, (op, grid, err)
