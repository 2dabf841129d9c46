"""GPU checkpoint / resume through the C ABI (ps3d_gpu_save_state,
ps3d_gpu_load_state).

A fresh context that loads a checkpoint holds the saved state bitwise, and a
run of 6 advances equals 3 advances, a checkpoint, the load and 3 more
advances bitwise: in both forms and both steppers, with a rolling-mean
prefactor (whose history the checkpoint carries) and with buoyancy.
Mismatched and damaged files are refused with a status.
"""
import numpy as np
import pytest

from ps3d_gb300 import Ps3dGpu, ic
from ps3d_gb300.solver import Ps3dError

pytestmark = pytest.mark.gpu

BOX = ic.BELTRAMI_BOX


def rel(x, y):
    return float(np.linalg.norm(x - y) / np.linalg.norm(y))


def _model(n, **kw):
    return Ps3dGpu(n, n, n, BOX["lower"], BOX["extent"], cflmax=0.5, **kw)


def _setup(m, n, buoyancy=False):
    vor, pert = ic.beltrami_plus_perturbation(n, n, n, seed=5, amplitude=1e-2)
    if buoyancy:
        b = ic.stratified_buoyancy(n, n, n, BOX["lower"], BOX["extent"], bfsq=2.0, amplitude=2e-2, seed=6)
        m.setup_fields(vor, pert, b)
    else:
        m.setup_fields(vor, pert)


@pytest.mark.parametrize("kw", [
    dict(precision="fp64"),
    dict(precision="mixed"),
    dict(precision="fp64", stepper="cn2"),
    dict(precision="mixed", pretype="roll-mean-max-strain", roll_mean_win_size=4),
    dict(precision="mixed", buoyancy=True),
], ids=["fp64", "mixed", "fp64-cn2", "mixed-rolling", "mixed-buoyancy"])
def test_resume_is_bitwise(kw, tmp_path):
    n = 32
    buoy = kw.get("buoyancy", False)
    a = _model(n, **kw)
    _setup(a, n, buoy)
    ta, da = a.advance_n(0.0, 6)

    b = _model(n, **kw)
    _setup(b, n, buoy)
    tb, _ = b.advance_n(0.0, 3)
    path = tmp_path / "state.bin"
    b.save_state(path, tb)
    saved = b.get("svor")
    b.close()

    c = _model(n, **kw)  # fresh context: nothing set up but the checkpoint
    t0 = c.load_state(path)
    assert t0 == tb
    assert np.array_equal(c.get("svor"), saved)
    tc, dc = c.advance_n(t0, 3)
    assert tc == ta, rel(np.array([tc]), np.array([ta]))
    assert np.array_equal(c.get("svor"), a.get("svor")), rel(c.get("svor"), a.get("svor"))
    if buoy:
        assert np.array_equal(c.get("sbuoy"), a.get("sbuoy"))
    for x, y in zip(dc, da[3:]):
        for key in ("dt", "ke", "rmv"):
            assert x[key] == y[key], key


def test_mismatched_and_damaged_checkpoints_are_refused(tmp_path):
    a = _model(32, precision="mixed")
    _setup(a, 32)
    path = tmp_path / "s.bin"
    a.save_state(path, 0.0)
    for other in (_model(16, precision="mixed"), _model(32, precision="fp64"), _model(32, precision="mixed", nnu=2)):
        with pytest.raises(Ps3dError):
            other.load_state(path)
    with pytest.raises(Ps3dError):
        a.load_state(tmp_path / "missing.bin")
    raw = path.read_bytes()
    (tmp_path / "short.bin").write_bytes(raw[: len(raw) // 2])
    with pytest.raises(Ps3dError):
        a.load_state(tmp_path / "short.bin")
    (tmp_path / "bad.bin").write_bytes(b"XXXXXXXX" + raw[8:])
    with pytest.raises(Ps3dError):
        a.load_state(tmp_path / "bad.bin")
    # rolling-mean ring indices outside 1..len (header: int32 roll_len at
    # byte 36, rollb_len 40, roll_inew 48, roll_iold 52, rollb_inew 60,
    # rollb_iold 64) are refused before anything is read into the context
    roll_len = int(np.frombuffer(raw[36:40], dtype=np.int32)[0])
    rollb_len = int(np.frombuffer(raw[40:44], dtype=np.int32)[0])
    for off, val in ((48, roll_len + 1), (52, 0), (60, rollb_len + 1), (64, -3)):
        patched = bytearray(raw)
        patched[off:off + 4] = np.int32(val).tobytes()
        (tmp_path / "idx.bin").write_bytes(bytes(patched))
        with pytest.raises(Ps3dError) as e:
            a.load_state(tmp_path / "idx.bin")
        assert e.value.code == 1, (off, val, e.value.code)  # PS3D_ERR_INVALID_ARG
    # the context still works after the refusals
    t, _ = a.advance(0.0)
    assert t > 0.0
