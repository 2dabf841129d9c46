"""GB300 (sm_103a) implementation of the ps3d vorticity right-hand side and
time steppers behind a C ABI (include/ps3d_gpu.h, libps3d_gpu.so).

    from ps3d_gb300 import Ps3dGpu
    m = Ps3dGpu(nx, ny, nz, lower, extent, precision="fp64")
    m.setup_fields(vor_phys)
    t, diag = m.advance(0.0)
"""
from .solver import Ps3dGpu, Ps3dError, batch_advance, make_config  # noqa: F401
from . import ic  # noqa: F401

__all__ = ["Ps3dGpu", "Ps3dError", "batch_advance", "make_config", "ic"]
