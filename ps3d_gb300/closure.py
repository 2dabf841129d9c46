"""Learned sub-grid closure for coarse runs (no counterpart in the reference).

The reference's only sub-grid model is the horizontal hyperdiffusion set up
by init_diffusion (inversion_utils.f90:124-218).  Here a coarse run may also
carry a small convolution network (libps3d_gpu.so, closure.cu) that adds a
vorticity-tendency correction to svorts at each advance; with no network
attached the run is the plain hyperdiffusive method.

Training data come from fine runs (FP64 or the mixed form, which stays
within 1e-6 of it): at a fine state omega_f, the target is the exact
sub-grid tendency

    target = cut(T_f(omega_f)) - T_c(cut(omega_f))

where T is the projected vorticity tendency (`source`, inversion.f90:298-388)
on each grid and `cut` is the sharp spectral truncation of the mixed-spectral
representation to the coarse grid (`spectral_cut`).  The network sees the
coarse run's physical vorticity and velocity (each over its rms) and is
trained to the physical target (over ct * <|omega|^2>).
"""
import ctypes

import numpy as np

from . import _lib

NPARAM = 63171
ENGINES = ("mma", "tcgen05")
_fp = ctypes.POINTER(ctypes.c_float)
_dp = ctypes.POINTER(ctypes.c_double)


class ClosureError(RuntimeError):
    pass


def _d(a):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_dp)


def _f(a):
    assert a.dtype == np.float32 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_fp)


class Closure:
    """One closure network for a grid of nx x ny x (nz+1) points on a device,
    with room for `max_samples` training samples in device memory."""

    def __init__(self, nx, ny, nz, max_samples=0, device=0, seed=0):
        self.nx, self.ny, self.nz = nx, ny, nz
        self.L = _lib.lib()
        self._h = ctypes.c_void_p()
        rc = self.L.ps3d_closure_create(nx, ny, nz, max_samples, device, seed, ctypes.byref(self._h))
        if rc != 0:
            raise ClosureError(f"{_lib.ERRORS.get(rc, rc)}: ps3d_closure_create")

    @property
    def handle(self):
        return self._h

    @property
    def shape(self):
        return (3, self.nx, self.ny, self.nz + 1)

    @property
    def npts(self):
        return self.nx * self.ny * (self.nz + 1)

    def _chk(self, rc):
        if rc != 0:
            msg = self.L.ps3d_closure_last_error(self._h).decode() if self._h else ""
            raise ClosureError(f"{_lib.ERRORS.get(rc, rc)}: {msg}")

    def close(self):
        if self._h:
            self._chk(self.L.ps3d_closure_destroy(self._h))
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def get_params(self):
        p = np.zeros(NPARAM, dtype=np.float32)
        self._chk(self.L.ps3d_closure_get_params(self._h, _f(p)))
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.shape == (NPARAM,)
        self._chk(self.L.ps3d_closure_set_params(self._h, _f(p)))

    @property
    def scale(self):
        v = ctypes.c_double()
        self._chk(self.L.ps3d_closure_get_scale(self._h, ctypes.byref(v)))
        return v.value

    @scale.setter
    def scale(self, ct):
        self._chk(self.L.ps3d_closure_set_scale(self._h, float(ct)))

    def _field(self, a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        assert a.shape == self.shape, (a.shape, self.shape)
        return a

    def add_sample(self, vor, vel, target):
        vor, vel, target = self._field(vor), self._field(vel), self._field(target)
        self._chk(self.L.ps3d_closure_add_sample(self._h, _d(vor), _d(vel), _d(target)))

    @property
    def num_samples(self):
        n = ctypes.c_int()
        self._chk(self.L.ps3d_closure_num_samples(self._h, ctypes.byref(n)))
        return n.value

    def train(self, iters, lr0=2e-3, lr1=1e-4, seed=0):
        """iters Adam steps; returns the per-step normalised loss."""
        loss = np.zeros(max(iters, 1))
        self._chk(self.L.ps3d_closure_train(self._h, int(iters), lr0, lr1, seed, _d(loss)))
        return loss[:iters]

    def predict(self, vor, vel):
        vor, vel = self._field(vor), self._field(vel)
        out = np.zeros(self.shape)
        self._chk(self.L.ps3d_closure_predict(self._h, _d(vor), _d(vel), _d(out)))
        return out

    @property
    def engine(self):
        """"mma" (warp-level mma.sync) or "tcgen05" (inference engine)"""
        e = ctypes.c_int()
        self._chk(self.L.ps3d_closure_get_engine(self._h, ctypes.byref(e)))
        return ENGINES[e.value]

    @engine.setter
    def engine(self, name):
        self._chk(self.L.ps3d_closure_set_engine(self._h, ENGINES.index(name)))

    def check(self):
        """raise if a bounded device wait of the tcgen05 engine ran out"""
        self._chk(self.L.ps3d_closure_check(self._h))

    def time_forward(self, reps=20):
        """device ms of one forward pass over the last predict's input"""
        ms = ctypes.c_double()
        self._chk(self.L.ps3d_closure_time_forward(self._h, int(reps), ctypes.byref(ms)))
        return ms.value

    def gradients(self, sample):
        """(normalised prediction (3, npts) FP32, parameter gradients, loss)
        of stored sample `sample`, without an update."""
        out = np.zeros((3, self.npts), dtype=np.float32)
        grad = np.zeros(NPARAM, dtype=np.float32)
        loss = ctypes.c_double()
        self._chk(self.L.ps3d_closure_gradients(self._h, int(sample), _f(out), _f(grad), ctypes.byref(loss)))
        return out, grad, loss.value


EVERY_STAGE, CLIP, WALLS = 1, 2, 4


def attach(model, closure, every_stage=False, clip=False, walls=False):
    """Attach `closure` to a Ps3dGpu model (None detaches: plain
    hyperdiffusion); the options are the PS3D_CLOSURE_* flags."""
    h = closure.handle if closure is not None else None
    flags = (EVERY_STAGE if every_stage else 0) | (CLIP if clip else 0) | (WALLS if walls else 0)
    model._chk(model.L.ps3d_gpu_set_closure(model._h, h, flags))


# ----------------------------------------------------------------- layout
NTAP = 27
LAYERS = ((6, 32), (32, 32), (32, 32), (32, 3))
# channels the kernels compute with (inputs padded to 16, the output to 8)
PADDED = ((16, 32), (32, 32), (32, 32), (32, 8))


def forward_flops(npts, padded=False):
    """multiply-add flops (2 per MAC) of one forward pass over npts points"""
    return 2.0 * npts * NTAP * sum(ci * co for ci, co in (PADDED if padded else LAYERS))


def param_views(p):
    """[(W[27, cin, cout], b[cout]) per layer] views of a parameter vector."""
    out, o = [], 0
    for cin, cout in LAYERS:
        w = p[o:o + NTAP * cin * cout].reshape(NTAP, cin, cout)
        o += NTAP * cin * cout
        b = p[o:o + cout]
        o += cout
        out.append((w, b))
    assert o == NPARAM
    return out


# ---------------------------------------------------------- spectral cut
def _horizontal_index(nf, nc):
    """Source slots in a length-nf Hermitian array (stafft.f90:55-58: slot 0
    the mean, slot k the cosine of mode k, slot n-k its sine) for the slots of
    a length-nc array, modes |k| < nc/2 (the coarse Nyquist slot dropped)."""
    h = nc // 2
    src = np.zeros(nc, dtype=np.int64)
    keep = np.ones(nc, dtype=bool)
    for k in range(1, h):
        src[k] = k
        src[nc - k] = nf - k
    src[h] = 0
    keep[h] = False
    return src, keep


def spectral_cut(f, nxc, nyc, nzc):
    """Sharp spectral truncation of a mixed-spectral field (..., nxf, nyf,
    nzf+1) to (..., nxc, nyc, nzc+1).

    Horizontal slots keep the modes |k| < n_c/2; the interior sine modes keep
    1..nzc-1; the wall rows (semi-spectral) carry over.  Every transform of
    the reference is scaled by sqrt(n) (stafft.f90:277, the orthonormal DST),
    so the kept coefficients are multiplied by sqrt(n_c/n_f) per transformed
    direction."""
    nxf, nyf, nzf = f.shape[-3], f.shape[-2], f.shape[-1] - 1
    assert nxc <= nxf and nyc <= nyf and nzc <= nzf
    sx, kx = _horizontal_index(nxf, nxc)
    sy, ky = _horizontal_index(nyf, nyc)
    g = f[..., sx, :, :][..., :, sy, :]
    g = g * (kx[:, None, None] & ky[None, :, None])
    hs = np.sqrt((nxc / nxf) * (nyc / nyf))
    out = np.empty(f.shape[:-3] + (nxc, nyc, nzc + 1))
    out[..., 0] = g[..., 0] * hs
    out[..., nzc] = g[..., nzf] * hs
    out[..., 1:nzc] = g[..., 1:nzc] * (hs * np.sqrt(nzc / nzf))
    return out


def subgrid_sample(fine, coarse):
    """(vor_c, vel_c, target) at the fine model's current state.

    fine, coarse: Ps3dGpu models on the same box; the coarse model must have
    no closure attached (its tendency is the plain coarse tendency).  The
    coarse model's state is overwritten with cut(svor_f)."""
    nxc, nyc, nzc = coarse.nx, coarse.ny, coarse.nz
    fine.vor2vel()
    fine.source()
    svor_c = spectral_cut(fine.get("svor"), nxc, nyc, nzc)
    ts_cut = spectral_cut(fine.get("svorts"), nxc, nyc, nzc)
    coarse.set("svor", svor_c)
    coarse.vor2vel()
    coarse.source()
    target_s = ts_cut - coarse.get("svorts")
    target = np.stack([coarse.combine_physical(target_s[k]) for k in range(3)])
    return coarse.get("vor"), coarse.get("vel"), target


def shell_error(e_model, e_truth, kmax=21):
    """max and mean over shells 1..kmax of |E_model - E_truth| / E_truth"""
    k = np.arange(1, kmax + 1)
    r = np.abs(e_model[k] - e_truth[k]) / np.abs(e_truth[k])
    return float(r.max()), float(r.mean())
