"""Compiled hosts of the C ABI driving real GPU steps.

tests/c_driver.c is the plain-C99 host (the calls a C or Fortran driver
makes: create, setup_fields, advance, save_state, destroy).  Here it must take
the device path: two FP64 steps of a 32^3 Beltrami run, a checkpoint written,
the energy series printed, and that series must agree with the same run
driven through the Python mirror to 1e-12 (the Beltrami field is evaluated by
the C library's sin/cos on one side and numpy's on the other, so the two
inputs agree to rounding, not bitwise).
"""
import os
import re
import shutil
import subprocess

import numpy as np
import pytest

from ps3d_gb300 import Ps3dGpu, _lib, build, ic

pytestmark = pytest.mark.gpu

TESTS = os.path.dirname(os.path.abspath(__file__))
INCLUDE = os.path.join(os.path.dirname(TESTS), "include")


def _compile_c_driver(tmp_path):
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("no C compiler")
    _lib.lib()
    exe = str(tmp_path / "c_driver")
    libdir = os.path.dirname(build.LIB)
    cmd = [gcc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-O1", "-I", INCLUDE, os.path.join(TESTS, "c_driver.c"),
           "-o", exe, "-L", libdir, "-lps3d_gpu", "-lm", "-Wl,-rpath," + libdir]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_c_driver_takes_the_device_path(tmp_path):
    exe = _compile_c_driver(tmp_path)
    ckpt = tmp_path / "state.bin"
    n, steps = 32, 2
    r = subprocess.run([exe, str(n), str(steps), str(ckpt)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    lines = r.stdout.splitlines()
    assert "no CUDA device" not in r.stdout and "NO_DEVICE" not in r.stdout.upper(), r.stdout
    head = re.match(r"c_driver: (\d+)\^3, te ([-\d.eE+]+), en ([-\d.eE+]+)", lines[0])
    assert head, lines[0]
    series = [re.match(r"c_driver: t ([-\d.eE+]+) dt ([-\d.eE+]+) ke ([-\d.eE+]+) en ([-\d.eE+]+) "
                       r"hel ([-\d.eE+]+)", s) for s in lines[1:]]
    assert len(series) == steps and all(series), lines
    assert ckpt.exists() and ckpt.stat().st_size > 3 * n * n * (n + 1) * 8

    # the same run through the Python mirror of the ABI
    lo, ex = ic.BELTRAMI_BOX["lower"], ic.BELTRAMI_BOX["extent"]
    vor = ic.beltrami_vorticity(n, n, n, lo, ex)
    g = Ps3dGpu(n, n, n, lo, ex, cflmax=0.5)
    te, en = g.setup_fields(vor, None)
    assert abs(te - float(head.group(2))) <= 1e-12 * abs(te)
    assert abs(en - float(head.group(3))) <= 1e-12 * abs(en)
    t = 0.0
    for s in range(steps):
        t, d = g.advance(t)
        got = [float(series[s].group(i)) for i in range(1, 6)]
        want = [t, d["dt"], d["ke"], d["en"], d["hel"]]
        # the driver prints t and dt with 6 decimals, ke, en and hel with 12
        for i, printed in enumerate((6, 6, 12, 12, 12)):
            assert abs(got[i] - want[i]) <= 1e-12 * abs(want[i]) + 0.5 * 10.0 ** -printed, (s, i, got, want)

    # the checkpoint the C host wrote resumes in a Python context
    h = Ps3dGpu(n, n, n, lo, ex, cflmax=0.5)
    t_c = h.load_state(ckpt)
    assert abs(t_c - t) <= 1e-14 * t
    svor_c, svor_p = h.get("svor"), g.get("svor")
    assert np.linalg.norm(svor_c - svor_p) <= 1e-12 * np.linalg.norm(svor_p)
