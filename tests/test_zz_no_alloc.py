"""ps3d_gpu_energy_series_noalloc: the energy series computed from device
arrays the caller owns, with no allocation inside the library.

The caller here plays the role of a driver that manages its own device
memory: it allocates the vel/vor device arrays and the 3-double output with
the CUDA runtime itself.  The result must match ps3d_gpu_energy_series of a
regular context on the same fields, on two calls in a row (the second with
different fields, so a stale scratch array would show), in the reference
layout (pitch nz+1, legacy default stream), in a padded layout (pitch nz+8,
padding rows filled with NaN, which the reduction must not read) on a stream
the caller created, and at the largest grid the scratch array admits.

The file is named so that pytest collects it last: it drives the CUDA
runtime directly with device memory of its own, outside any library
context, so if it fails, a run that stops at the first failure
(`pytest -x`) has already run every other test.
"""
import ctypes

import numpy as np
import pytest

from ps3d_gb300 import Ps3dGpu, _lib, ic

pytestmark = pytest.mark.gpu

MAX_COLUMNS = 524288  # nx*ny admitted by the scratch array (65536 blocks x 8 columns)


def _cudart():
    for name in ("libcudart.so", "libcudart.so.13", "/usr/local/cuda/lib64/libcudart.so"):
        try:
            return ctypes.CDLL(name)
        except OSError:
            continue
    pytest.skip("libcudart not found")


def _to_device(rt, a, ptrs):
    p = ctypes.c_void_p()
    assert rt.cudaMalloc(ctypes.byref(p), ctypes.c_size_t(a.nbytes)) == 0
    ptrs.append(p)
    assert rt.cudaMemcpy(p, a.ctypes.data_as(ctypes.c_void_p), ctypes.c_size_t(a.nbytes), 1) == 0
    return p


def _repitch(f, pitch):
    """(3, nx, ny, nz+1) host field -> (3, nx, ny, pitch), padding rows NaN."""
    out = np.full(f.shape[:3] + (pitch,), np.nan)
    out[..., : f.shape[3]] = f
    return np.ascontiguousarray(out)


def _noalloc(rt, L, vel, vor, nx, ny, nz, pitch, stream, out, ptrs):
    dvel, dvor = _to_device(rt, vel, ptrs), _to_device(rt, vor, ptrs)
    nfield = pitch * nx * ny
    rc = L.ps3d_gpu_energy_series_noalloc(dvel, dvor, nx, ny, nz, pitch, nfield, stream, out)
    assert rc == 0, rc
    if stream is None:
        assert rt.cudaDeviceSynchronize() == 0
    else:
        assert rt.cudaStreamSynchronize(stream) == 0
    got = np.zeros(3)
    assert rt.cudaMemcpy(got.ctypes.data_as(ctypes.c_void_p), out, ctypes.c_size_t(24), 2) == 0
    return got


def _case(rt, L, nx, ny, nz, pads, stream):
    lo, ex = ic.BELTRAMI_BOX["lower"], ic.BELTRAMI_BOX["extent"]
    vor0, pert = ic.beltrami_plus_perturbation(nx, ny, nz, seed=3)
    g = Ps3dGpu(nx, ny, nz, lo, ex)
    out = ctypes.c_void_p()
    assert rt.cudaMalloc(ctypes.byref(out), ctypes.c_size_t(24)) == 0
    ptrs = [out]
    try:
        for call, scale in enumerate((1.0, 0.5)):
            g.setup_fields(vor0 * scale, pert * scale)
            ref = np.array(g.energy_series())
            vel = np.ascontiguousarray(g.get("vel"))
            vor = np.ascontiguousarray(g.get("vor"))
            for pad in pads:
                pitch = nz + 1 + pad
                got = _noalloc(rt, L, _repitch(vel, pitch), _repitch(vor, pitch), nx, ny, nz, pitch, stream,
                               out, ptrs)
                np.testing.assert_allclose(got, ref, rtol=1e-12, atol=0, err_msg=f"call {call}, pitch {pitch}")
    finally:
        for p in ptrs:
            rt.cudaFree(p)
        g.close()


def test_energy_series_noalloc_matches_context_path():
    rt = _cudart()
    L = _lib.lib()
    _case(rt, L, 32, 32, 32, pads=(0,), stream=None)


def test_energy_series_noalloc_padded_layout_on_a_created_stream():
    rt = _cudart()
    L = _lib.lib()
    stream = ctypes.c_void_p()
    assert rt.cudaStreamCreate(ctypes.byref(stream)) == 0
    try:
        _case(rt, L, 32, 16, 16, pads=(7,), stream=stream)
    finally:
        rt.cudaStreamDestroy(stream)


def test_energy_series_noalloc_at_the_scratch_limit_and_beyond():
    rt = _cudart()
    L = _lib.lib()
    _case(rt, L, 1024, 512, 8, pads=(0,), stream=None)  # nx*ny = MAX_COLUMNS
    out = ctypes.c_void_p()
    assert rt.cudaMalloc(ctypes.byref(out), ctypes.c_size_t(24)) == 0
    try:
        # refused before any launch: one column pair beyond the scratch
        # capacity, a pitch below nz+1 or above INT_MAX, a component stride
        # below pitch*nx*ny (NULL field pointers are never dereferenced
        # because the checks come first; a dummy non-NULL value stands in)
        dummy = ctypes.c_void_p(256)
        f = L.ps3d_gpu_energy_series_noalloc
        assert f(dummy, dummy, 1024, 520, 8, 9, 9 * 1024 * 520, None, out) == 2
        assert f(dummy, dummy, 1024, 1024, 8, 9, 9 * 1024 * 1024, None, out) == 2
        assert f(dummy, dummy, 16, 16, 8, 8, 9 * 256, None, out) == 1
        assert f(dummy, dummy, 16, 16, 8, 2 ** 31, 2 ** 31 * 256, None, out) == 1
        assert f(dummy, dummy, 16, 16, 8, 9, 9 * 256 - 1, None, out) == 1
        assert MAX_COLUMNS == 1024 * 512
    finally:
        rt.cudaFree(out)
