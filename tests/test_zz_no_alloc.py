"""ps3d_gpu_energy_series_noalloc: the energy series computed from device
arrays the caller owns, with no allocation inside the library.

The caller here plays the role of a driver that manages its own device
memory: it allocates the vel/vor device arrays and the 3-double output with
the CUDA runtime itself, in the reference layout (pitch nz+1).  The result
must match ps3d_gpu_energy_series of a regular context on the same fields,
on two calls in a row (the second with different fields, so a stale scratch
array would show).  This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

from ps3d_gb300 import Ps3dGpu, _lib, ic

pytestmark = pytest.mark.gpu


def _cudart():
    for name in ("libcudart.so", "libcudart.so.13", "/usr/local/cuda/lib64/libcudart.so"):
        try:
            return ctypes.CDLL(name)
        except OSError:
            continue
    pytest.skip("libcudart not found")


def _to_device(rt, a):
    p = ctypes.c_void_p()
    assert rt.cudaMalloc(ctypes.byref(p), ctypes.c_size_t(a.nbytes)) == 0
    assert rt.cudaMemcpy(p, a.ctypes.data_as(ctypes.c_void_p), ctypes.c_size_t(a.nbytes), 1) == 0
    return p


def test_energy_series_noalloc_matches_context_path():
    rt = _cudart()
    L = _lib.lib()
    n = 32
    lo, ex = ic.BELTRAMI_BOX["lower"], ic.BELTRAMI_BOX["extent"]
    vor0, pert = ic.beltrami_plus_perturbation(n, n, n, seed=3)
    g = Ps3dGpu(n, n, n, lo, ex)
    out = ctypes.c_void_p()
    assert rt.cudaMalloc(ctypes.byref(out), ctypes.c_size_t(24)) == 0
    ptrs = [out]
    try:
        for call, scale in enumerate((1.0, 0.5)):
            g.setup_fields(vor0 * scale, pert * scale)
            ref = np.array(g.energy_series())
            vel = np.ascontiguousarray(g.get("vel"))
            vor = np.ascontiguousarray(g.get("vor"))
            dvel, dvor = _to_device(rt, vel), _to_device(rt, vor)
            ptrs += [dvel, dvor]
            nfield = n * n * (n + 1)
            rc = L.ps3d_gpu_energy_series_noalloc(dvel, dvor, n, n, n, n + 1, nfield, None, out)
            assert rc == 0, (call, rc)
            assert rt.cudaDeviceSynchronize() == 0
            got = np.zeros(3)
            assert rt.cudaMemcpy(got.ctypes.data_as(ctypes.c_void_p), out, ctypes.c_size_t(24), 2) == 0
            np.testing.assert_allclose(got, ref, rtol=1e-12, atol=0, err_msg=f"call {call}")
        # sizes beyond the scratch capacity are refused before any launch
        assert L.ps3d_gpu_energy_series_noalloc(ptrs[1], ptrs[2], 1024, 1024, 8, 9, 9 * 1024 * 1024,
                                                None, out) == 2
    finally:
        for p in ptrs:
            rt.cudaFree(p)
        g.close()
