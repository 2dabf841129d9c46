"""GPU checks of the learned sub-grid closure (closure.cu) through the C ABI.

The network's BF16 tensor-core kernels are compared with a PyTorch
reference of the same network (conv3d with periodic x, y and zero z
padding, exact GELU): in FP64 with the library's BF16 roundings emulated
(tight), and in plain FP64 (loose: BF16 activations).  The Adam update is
checked against its formula; attaching a network whose parameters are zero
must leave a run bitwise unchanged; the FP64 tendency with a closure
attached must differ from the plain one by exactly the decomposed
correction; captured steps must equal host-driven ones.
"""
import numpy as np
import pytest

from ps3d_gb300 import Ps3dGpu, ic
from ps3d_gb300.closure import NPARAM, Closure, attach, param_views, spectral_cut, subgrid_sample

torch = pytest.importorskip("torch")
F = torch.nn.functional

pytestmark = pytest.mark.gpu

LO, EX = ic.BELTRAMI_BOX["lower"], ic.BELTRAMI_BOX["extent"]
# tolerances: relative L2 against the reference with the BF16 roundings
# emulated / against plain FP64
TOL_EMU_OUT, TOL_FP64_OUT = 5e-3, 3e-2
TOL_EMU_GRAD, TOL_EMU_LOSS = 3e-2, 1e-3


def bf16(x):
    return x.to(torch.bfloat16).to(x.dtype)


def conv(a, W, b):
    cin, cout = W.shape[1], W.shape[2]
    w = W.reshape(3, 3, 3, cin, cout).permute(4, 3, 0, 1, 2).contiguous()
    ap = F.pad(a, (0, 0, 1, 1, 1, 1), mode="circular")
    ap = F.pad(ap, (1, 1, 0, 0, 0, 0))
    return F.conv3d(ap, w, b)


def reference(params, vor, vel, emulate):
    """network output (1, 3, nx, ny, nz+1), FP64, and the parameter tensors"""
    npts = vor[0].size
    w2 = float(np.sum(vor * vor)) / npts
    u2 = float(np.sum(vel * vel)) / npts
    x = np.concatenate([vor / np.sqrt(w2), vel / np.sqrt(u2)])[None]
    a = torch.tensor(x, dtype=torch.float64)
    if emulate:
        a = bf16(a)
    tens = []
    for l, (W, b) in enumerate(param_views(params.astype(np.float64))):
        Wt = torch.tensor(W, dtype=torch.float64, requires_grad=True)
        bt = torch.tensor(b, dtype=torch.float64, requires_grad=True)
        tens += [Wt, bt]
        z = conv(a, bf16(Wt) if emulate else Wt, bt)
        if l < 3:
            if emulate:
                z = bf16(z)
            a = F.gelu(z)
            if emulate:
                a = bf16(a)
        else:
            a = z
    return a, tens, w2


def random_fields(shape, seed):
    rng = np.random.default_rng(seed)
    return [rng.standard_normal((3,) + shape) * s for s in (2.0, 0.5, 1e-2)]


def boosted_params(cl):
    p = cl.get_params()
    views = param_views(p)
    views[-1][0][...] *= 10.0  # an output of order one
    rng = np.random.default_rng(5)
    for _, b in views:
        b[...] = 0.1 * rng.standard_normal(b.shape)
    return p


@pytest.mark.parametrize("dims", [(16, 16, 16), (16, 8, 32)])
def test_forward_and_gradients_match_torch(dims):
    nx, ny, nz = dims
    shape = (nx, ny, nz + 1)
    vor, vel, tgt = random_fields(shape, 1)
    cl = Closure(nx, ny, nz, max_samples=1, seed=3)
    p = boosted_params(cl)
    cl.set_params(p)
    ct = 0.01
    cl.scale = ct
    cl.add_sample(vor, vel, tgt)
    out, grad, loss = cl.gradients(0)
    out = out.reshape((3,) + shape)

    ref, tens, w2 = reference(p, vor, vel, emulate=True)
    r = ref[0].detach().numpy()
    e = np.linalg.norm(out - r) / np.linalg.norm(r)
    assert e < TOL_EMU_OUT, e
    ref64, _, _ = reference(p, vor, vel, emulate=False)
    r64 = ref64[0].detach().numpy()
    e64 = np.linalg.norm(out - r64) / np.linalg.norm(r64)
    assert e64 < TOL_FP64_OUT, e64

    tn = torch.tensor(tgt / (ct * w2), dtype=torch.float64)[None]
    lref = torch.mean((ref - tn) ** 2)
    lref.backward()
    assert abs(loss - float(lref)) < TOL_EMU_LOSS * float(lref)
    o = 0
    for l, (W, b) in enumerate(param_views(np.arange(NPARAM))):
        gw = grad[o:o + W.size]
        rw = tens[2 * l].grad.numpy().ravel()
        o += W.size
        gb = grad[o:o + b.size]
        rb = tens[2 * l + 1].grad.numpy().ravel()
        o += b.size
        ew = np.linalg.norm(gw - rw) / np.linalg.norm(rw)
        eb = np.linalg.norm(gb - rb) / np.linalg.norm(rb)
        assert ew < TOL_EMU_GRAD, (l, ew)
        assert eb < TOL_EMU_GRAD, (l, eb)
    cl.close()


def test_adam_step_follows_its_formula():
    shape = (16, 16, 17)
    vor, vel, tgt = random_fields(shape, 2)
    cl = Closure(16, 16, 16, max_samples=1, seed=4)
    cl.set_params(boosted_params(cl))
    cl.scale = 0.01
    cl.add_sample(vor, vel, tgt)
    p0 = cl.get_params()
    _, g, _ = cl.gradients(0)
    lr = 1e-3
    cl.train(1, lr, lr)
    p1 = cl.get_params()
    # first Adam step: m_hat = g, v_hat = g^2
    g = g.astype(np.float64)
    expect = p0 - lr * g / (np.sqrt(g * g) + 1e-8)
    assert np.max(np.abs(p1 - expect)) < 2e-6
    cl.close()


def test_training_reduces_the_loss_on_a_teacher_network():
    shape = (16, 16, 17)
    teacher = Closure(16, 16, 16, seed=11)
    teacher.set_params(boosted_params(teacher))
    teacher.scale = 1.0
    student = Closure(16, 16, 16, max_samples=4, seed=12)
    student.scale = 1.0
    for s in range(4):
        vor, vel, _ = random_fields(shape, 20 + s)
        student.add_sample(vor, vel, teacher.predict(vor, vel))
    loss = student.train(300, 3e-3, 3e-4, seed=5)
    assert np.all(np.isfinite(loss))
    assert loss[-20:].mean() < 0.5 * loss[:4].mean(), (loss[:4].mean(), loss[-20:].mean())
    teacher.close()
    student.close()


def _pair(n, precision):
    a = Ps3dGpu(n, n, n, LO, EX, precision=precision, cflmax=0.5)
    b = Ps3dGpu(n, n, n, LO, EX, precision=precision, cflmax=0.5)
    vor, pert = ic.beltrami_plus_perturbation(n, n, n, seed=3, amplitude=1e-2)
    a.setup_fields(vor, pert)
    b.setup_fields(vor, pert)
    return a, b


def test_zero_network_leaves_the_run_unchanged():
    a, b = _pair(32, "mixed")
    cl = Closure(32, 32, 32, seed=1)
    cl.set_params(np.zeros(NPARAM, dtype=np.float32))
    cl.scale = 1.0
    attach(b, cl)
    ta = tb = 0.0
    for _ in range(3):
        ta, _ = a.advance(ta)
        tb, _ = b.advance(tb)
    assert ta == tb
    assert np.array_equal(a.get("svor"), b.get("svor"))
    attach(b, None)
    cl.close()


def test_fp64_tendency_gains_the_decomposed_correction():
    a, b = _pair(32, "fp64")
    cl = Closure(32, 32, 32, seed=2)
    cl.set_params(boosted_params(cl))
    cl.scale = 0.05
    attach(b, cl)
    for m in (a, b):
        m.vor2vel()
        m.source()
    corr = cl.predict(b.get("vor"), b.get("vel"))
    expect = np.stack([a.decompose_physical(corr[k]) for k in range(3)])
    diff = b.get("svorts") - a.get("svorts")
    assert np.linalg.norm(expect) > 1e-3 * np.linalg.norm(a.get("svorts"))
    err = np.linalg.norm(diff - expect) / np.linalg.norm(expect)
    assert err < 1e-10, err
    attach(b, None)
    cl.close()


def test_clip_and_wall_options_shape_the_correction():
    a, b = _pair(32, "fp64")
    cl = Closure(32, 32, 32, seed=2)
    cl.set_params(boosted_params(cl))
    cl.scale = 0.05
    attach(b, cl, clip=True, walls=True)
    for m in (a, b):
        m.vor2vel()
        m.source()
    vor = b.get("vor")
    raw = cl.predict(vor, b.get("vel"))
    corr = raw.copy()
    corr[0:2, :, :, 0] = 0.0
    corr[0:2, :, :, -1] = 0.0
    w = np.sum(vor * corr, axis=0)
    # points whose vor . corr lies within rounding of zero may fall either way
    ambiguous = np.abs(w) <= 1e-9 * np.sqrt(np.sum(vor * vor, axis=0) * np.sum(corr * corr, axis=0))
    corr[:, w > 0.0] = 0.0
    diff = b.get("svorts") - a.get("svorts")
    added = np.stack([a.combine_physical(diff[k]) for k in range(3)])  # the correction the run added
    mism = np.max(np.abs(added - corr), axis=0) > 1e-8 * np.max(np.abs(raw))
    bad = mism & ~ambiguous
    assert not np.any(bad), (int(bad.sum()), int(mism.sum()), int(ambiguous.sum()))
    assert np.all(np.abs(added[0:2, :, :, 0]) < 1e-8 * np.max(np.abs(raw)))
    assert 0.1 < np.mean(w > 0.0) < 0.9  # the clip removed a part, not all
    attach(b, None)
    cl.close()


def test_closure_serves_one_context_and_detaches():
    a, b = _pair(32, "mixed")
    cl = Closure(32, 32, 32, seed=2)
    with pytest.raises(Exception):
        attach(a, cl)  # output scale not set yet
    cl.scale = 1.0
    attach(a, cl)
    with pytest.raises(Exception):
        attach(b, cl)  # attached elsewhere
    with pytest.raises(Exception):
        cl.close()     # still attached
    attach(a, None)
    attach(b, cl)
    attach(b, None)
    other = Closure(16, 16, 16, seed=2)
    other.scale = 1.0
    with pytest.raises(Exception):
        attach(a, other)  # grid differs
    cl.close()
    other.close()


@pytest.mark.parametrize("every_stage", [False, True])
def test_captured_steps_with_closure_match_host_driven(every_stage):
    a, b = _pair(32, "mixed")
    cl1 = Closure(32, 32, 32, seed=9)
    cl1.set_params(boosted_params(cl1))
    cl1.scale = 0.02
    cl2 = Closure(32, 32, 32, seed=9)
    cl2.set_params(cl1.get_params())
    cl2.scale = 0.02
    attach(a, cl1, every_stage)
    attach(b, cl2, every_stage)
    ta, _ = a.advance_n(0.0, 4)
    tb, _, _ = b.advance_graph(0.0, 4)
    assert ta == tb
    assert np.array_equal(a.get("svor"), b.get("svor"))
    attach(a, None)
    attach(b, None)
    cl1.close()
    cl2.close()


def test_subgrid_sample_of_a_resolved_flow_is_small():
    nf, nc = 64, 32
    fine = Ps3dGpu(nf, nf, nf, LO, EX, precision="fp64", cflmax=0.5)
    coarse = Ps3dGpu(nc, nc, nc, LO, EX, precision="fp64", cflmax=0.5)
    vor, pert = ic.beltrami_plus_perturbation(nf, nf, nf, seed=4, amplitude=0.0)
    fine.setup_fields(vor, pert)
    vc, uc, tgt = subgrid_sample(fine, coarse)
    assert vc.shape == (3, nc, nc, nc + 1) and np.all(np.isfinite(tgt))
    # the Beltrami state is resolved on both grids: what remains is the
    # difference of the two grids' z finite differences
    coarse.set("svor", spectral_cut(fine.get("svor"), nc, nc, nc))
    coarse.vor2vel()
    assert np.allclose(coarse.get("vor"), vc)
    assert np.linalg.norm(tgt) < 0.1 * np.linalg.norm(vc) ** 2 / np.sqrt(vc[0].size)


@pytest.mark.parametrize("dims", [(16, 16, 16), (32, 16, 32), (64, 64, 64)])
def test_tcgen05_engine_matches_warp_engine_and_torch(dims):
    nx, ny, nz = dims
    shape = (nx, ny, nz + 1)
    vor, vel, _ = random_fields(shape, 7)
    cl = Closure(nx, ny, nz, seed=6)
    p = boosted_params(cl)
    cl.set_params(p)
    cl.scale = 1.0
    assert cl.engine == "tcgen05"  # the default where the grid allows it
    cl.engine = "mma"
    ref = cl.predict(vor, vel)
    cl.engine = "tcgen05"
    out = cl.predict(vor, vel)
    cl.check()
    err = np.linalg.norm(out - ref) / np.linalg.norm(ref)
    assert err < TOL_EMU_OUT, err
    w2 = float(np.sum(vor * vor)) / vor[0].size
    r, _, _ = reference(p, vor, vel, emulate=True)
    r = r[0].detach().numpy() * w2  # ct = 1: correction = output * <|vor|^2>
    e = np.linalg.norm(out - r) / np.linalg.norm(r)
    assert e < TOL_EMU_OUT, e
    cl.close()


def test_tcgen05_engine_in_a_run():
    a, b = _pair(32, "fp64")
    cl = Closure(32, 32, 32, seed=2)
    cl.set_params(boosted_params(cl))
    cl.scale = 0.05
    cl.engine = "tcgen05"
    attach(b, cl)
    for m in (a, b):
        m.vor2vel()
        m.source()
    cl.check()
    corr = cl.predict(b.get("vor"), b.get("vel"))
    expect = np.stack([a.decompose_physical(corr[k]) for k in range(3)])
    diff = b.get("svorts") - a.get("svorts")
    err = np.linalg.norm(diff - expect) / np.linalg.norm(expect)
    assert err < 1e-10, err
    attach(b, None)
    # captured steps with the tcgen05 engine equal host-driven ones
    c, d = _pair(32, "mixed")
    cl2 = Closure(32, 32, 32, seed=9)
    cl2.set_params(cl.get_params())
    cl2.scale = 0.05
    cl2.engine = "tcgen05"
    cl.set_params(cl2.get_params())
    attach(c, cl, every_stage=True)
    attach(d, cl2, every_stage=True)
    tc, _ = c.advance_n(0.0, 3)
    td, _, _ = d.advance_graph(0.0, 3)
    cl.check()
    cl2.check()
    assert tc == td
    assert np.array_equal(c.get("svor"), d.get("svor"))
    attach(c, None)
    attach(d, None)
    cl.close()
    cl2.close()
