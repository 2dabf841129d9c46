"""CPU-side checks of the C ABI: the library builds, loads and exports every
entry point include/ps3d_gpu.h declares; argument validation happens on the
host before any device call."""
import ctypes
import os
import re

import pytest

from ps3d_gb300 import _lib, build
from ps3d_gb300.solver import make_config

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "ps3d_gpu.h")


def declared():
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"\b(ps3d_(?:gpu|closure)_\w+)\s*\(", txt)))


def test_header_lists_match_binding():
    assert declared() == sorted(_lib.EXPORTS)


def test_library_exports_every_declared_symbol():
    L = _lib.lib()
    missing = [n for n in declared() if not hasattr(L, n)]
    assert not missing, missing


def test_library_is_built_for_sm_103a():
    # the build recipe pins one -gencode target
    assert build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]
    assert os.path.exists(build.LIB)


def test_strerror_codes():
    L = _lib.lib()
    for code in range(0, 9):
        assert L.ps3d_gpu_strerror(code)
    assert L.ps3d_gpu_strerror(999) == b"unknown status"


@pytest.mark.parametrize("dims", [(14, 32, 32), (32, 32, 15), (32, 22, 32), (4, 32, 32), (4096, 8, 8),
                                  (32, 32, 2048)])
def test_unsupported_sizes_rejected_before_device(dims):
    """Lengths must be even with factors 2, 3 and 5 only (the factorisation of
    stafft.f90:128-187), 8..2048 (z up to 1024 in FP64)."""
    L = _lib.lib()
    cfg = make_config(*dims, [0, 0, 0], [1, 1, 1])
    h = ctypes.c_void_p()
    assert L.ps3d_gpu_create(ctypes.byref(cfg), ctypes.byref(h)) == 2  # UNSUPPORTED_SIZE
    assert not h.value


@pytest.mark.parametrize("dims", [(30, 32, 32), (32, 32, 12), (48, 40, 24), (384, 8, 96)])
def test_mixed_radix_sizes_pass_the_size_check(dims):
    """n = 2^a 3^b 5^c passes the size check: without a device the call gets
    as far as the device query (NO_DEVICE); with one it creates a context."""
    L = _lib.lib()
    cfg = make_config(*dims, [0, 0, 0], [1, 1, 1])
    h = ctypes.c_void_p()
    rc = L.ps3d_gpu_create(ctypes.byref(cfg), ctypes.byref(h))
    assert rc in (0, 8), rc
    if rc == 0:
        L.ps3d_gpu_destroy(h)


def test_invalid_config_rejected():
    L = _lib.lib()
    h = ctypes.c_void_p()
    cfg = make_config(32, 32, 32, [0, 0, 0], [1, 1, 1], precision=7)
    assert L.ps3d_gpu_create(ctypes.byref(cfg), ctypes.byref(h)) == 1
    cfg = make_config(32, 32, 32, [0, 0, 0], [1, 0, 1])
    assert L.ps3d_gpu_create(ctypes.byref(cfg), ctypes.byref(h)) == 1
    assert L.ps3d_gpu_create(None, ctypes.byref(h)) == 1


def test_null_context_is_an_error_not_a_crash():
    L = _lib.lib()
    assert L.ps3d_gpu_vor2vel(None) == 1
    assert L.ps3d_gpu_destroy(None) == 0


def test_closure_and_checkpoint_entry_points_validate_on_the_host():
    L = _lib.lib()
    h = ctypes.c_void_p()
    # sizes are checked before any device call
    assert L.ps3d_closure_create(12, 16, 16, 0, 0, 0, ctypes.byref(h)) == 2
    assert L.ps3d_closure_create(16, 16, 16, -1, 0, 0, ctypes.byref(h)) in (1, 8)
    assert L.ps3d_closure_create(16, 16, 16, 0, 0, 0, None) == 1
    assert not h.value
    assert L.ps3d_closure_destroy(None) == 0
    assert L.ps3d_closure_set_scale(None, 1.0) == 1
    assert L.ps3d_closure_get_scale(None, None) == 1
    assert L.ps3d_closure_set_engine(None, 1) == 1
    assert L.ps3d_closure_num_samples(None, None) == 1
    assert L.ps3d_closure_last_error(None) == b""
    t = ctypes.c_double()
    assert L.ps3d_gpu_save_state(None, b"x", 0.0) == 1
    assert L.ps3d_gpu_load_state(None, b"x", ctypes.byref(t)) == 1
    assert L.ps3d_gpu_set_closure(None, None, 0) == 1


def test_c_driver_builds_and_runs_against_the_c_abi(tmp_path):
    """tests/c_driver.c uses the ABI from plain C99 (-Wall -Wextra -Werror):
    the header needs no C++, the library links, and without a device the
    driver ends cleanly with PS3D_ERR_NO_DEVICE (with one it runs two steps
    and writes a checkpoint)."""
    import shutil
    import subprocess
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("no C compiler")
    _lib.lib()  # built
    src = os.path.join(os.path.dirname(os.path.abspath(__file__)), "c_driver.c")
    exe = str(tmp_path / "c_driver")
    libdir = os.path.dirname(build.LIB)
    cmd = [gcc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-O1", "-I", os.path.dirname(HEADER), src,
           "-o", exe, "-L", libdir, "-lps3d_gpu", "-lm", "-Wl,-rpath," + libdir]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe, "16", "2", str(tmp_path / "state.bin")], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("c_driver:")
