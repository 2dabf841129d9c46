"""Host-side mirror of the reference's hot-path interface over the C ABI.

`Ps3dGpu` exposes the procedures of the reference's inversion and stepper
modules (vor2vel, source, adapt, step, advance, the transform helpers of
sta3dfft/inversion_utils) with the same argument meaning, acting on one GPU
context.  Fields are numpy arrays in the reference layout: a scalar field is
shaped (nx, ny, nz+1) in C order (z fastest), a vector field (3, nx, ny, nz+1).
Every call goes through libps3d_gpu.so; a non-zero status raises Ps3dError.
"""
import ctypes

import numpy as np

from . import _lib

PRETYPES = {"constant": 0, "vorch": 1, "bfmax": 2, "roll-mean-max-strain": 3,
            "max-strain": 4, "us-max-strain": 5, "roll-mean-bfmax": 6}
LENGTH_SCALES = {"Kolmogorov": 0, "geophysical": 1}
FILTERS = {"Hou & Li": 0, "2/3-rule": 1}
STEPPERS = {"impl-diff-rk4": 0, "cn2": 1}
PRECISIONS = {"fp64": 0, "mixed": 1}
FIELDS = {"svor": 0, "vor": 1, "vel": 2, "svel": 3, "svorts": 4,
          "sbuoy": 5, "buoy": 6, "sbuoys": 7}
SCALAR_FIELDS = ("sbuoy", "buoy", "sbuoys")
TABLES = {"k2l2": 0, "k2l2i": 1, "filt": 2, "green": 3, "phim": 4, "phip": 5,
          "thetam": 6, "thetap": 7, "dthetam": 8, "dthetap": 9, "gamtop": 10,
          "gambot": 11, "vhdis": 12, "rkx": 13, "rky": 14, "rkz": 15,
          "dphim": 16, "dphip": 17, "bhdis": 18, "bbarz": 19}
OPS = {"fftxyp2s": 0, "fftxys2p": 1, "diffx": 2, "diffy": 3, "fftsine": 4,
       "fftcosine": 5, "central_diffz": 6, "decompose_semi_spectral": 7,
       "combine_semi_spectral": 8, "decompose_physical": 9, "combine_physical": 10,
       "diffz": 11}

_dp = ctypes.POINTER(ctypes.c_double)


class Ps3dError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{_lib.ERRORS.get(code, code)}: {msg}")
        self.code = code


def _ptr(a):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_dp)


def make_config(nx, ny, nz, lower, extent, nnu=3, prediss=30.0, pretype="vorch",
                length_scale="Kolmogorov", filtering="Hou & Li", stepper="impl-diff-rk4",
                cflmax=0.8, alpha=0.1, time_limit=1.0e30, roll_mean_win_size=1000,
                hold_source=0, f_cor=(0.0, 0.0, 0.0), precision="fp64", device=0, nthreads=0,
                buoyancy=False, bfsq=None, buoy_nnu=3, buoy_prediss=30.0, buoy_pretype="bfmax",
                buoy_length_scale="Kolmogorov", buoy_roll_mean_win_size=1000):
    c = _lib.Config()
    c.nx, c.ny, c.nz, c.nnu = nx, ny, nz, nnu
    c.lower[:] = list(lower)
    c.extent[:] = list(extent)
    c.prediss = prediss
    c.pretype = PRETYPES[pretype] if isinstance(pretype, str) else int(pretype)
    c.length_scale = LENGTH_SCALES[length_scale] if isinstance(length_scale, str) else int(length_scale)
    c.filtering = FILTERS[filtering] if isinstance(filtering, str) else int(filtering)
    c.stepper = STEPPERS[stepper] if isinstance(stepper, str) else int(stepper)
    c.cflmax, c.alpha, c.time_limit = cflmax, alpha, time_limit
    c.roll_mean_win_size, c.nthreads, c.hold_source = roll_mean_win_size, nthreads, int(hold_source)
    c.f_cor[:] = list(f_cor)
    c.precision = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
    c.device = device
    c.buoyancy = int(bool(buoyancy))
    c.bfsq = 0.0 if bfsq is None else float(bfsq)
    c.bfsq_given = int(bfsq is not None)
    c.buoy_nnu, c.buoy_prediss = buoy_nnu, buoy_prediss
    c.buoy_pretype = PRETYPES[buoy_pretype] if isinstance(buoy_pretype, str) else int(buoy_pretype)
    c.buoy_length_scale = (LENGTH_SCALES[buoy_length_scale] if isinstance(buoy_length_scale, str)
                           else int(buoy_length_scale))
    c.buoy_roll_mean_win_size = buoy_roll_mean_win_size
    return c


class Ps3dGpu:
    """One GPU model of the ps3d hot path (the drop-in for the reference's
    inversion_mod / impl_rk4_mod / cn2_mod / advance_mod procedures)."""

    def __init__(self, nx, ny, nz, lower, extent, **kw):
        self.nx, self.ny, self.nz = nx, ny, nz
        self.precision = kw.get("precision", "fp64")
        self.cfg = make_config(nx, ny, nz, lower, extent, **kw)
        self.L = _lib.lib()
        self._h = ctypes.c_void_p()
        rc = self.L.ps3d_gpu_create(ctypes.byref(self.cfg), ctypes.byref(self._h))
        if rc != 0:
            raise Ps3dError(rc, self.L.ps3d_gpu_strerror(rc).decode())

    # ------------------------------------------------------------ plumbing
    def _chk(self, rc):
        if rc != 0:
            msg = self.L.ps3d_gpu_last_error(self._h).decode() if self._h else ""
            raise Ps3dError(rc, msg or self.L.ps3d_gpu_strerror(rc).decode())

    def close(self):
        if self._h:
            self.L.ps3d_gpu_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def shape(self):
        return (self.nx, self.ny, self.nz + 1)

    @property
    def device_bytes(self):
        return self.L.ps3d_gpu_device_bytes(self._h)

    @property
    def launch_count(self):
        return self.L.ps3d_gpu_launch_count(self._h)

    # ---------------------------------------------------- field operators
    def _op(self, name, a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        assert a.shape == self.shape, (a.shape, self.shape)
        out = np.zeros(self.shape)
        self._chk(self.L.ps3d_gpu_field_op(self._h, OPS[name], _ptr(a), _ptr(out)))
        return out

    def fftxyp2s(self, fp): return self._op("fftxyp2s", fp)
    def fftxys2p(self, fs): return self._op("fftxys2p", fs)
    def diffx(self, fs): return self._op("diffx", fs)
    def diffy(self, fs): return self._op("diffy", fs)
    def fftsine(self, fs): return self._op("fftsine", fs)
    def fftcosine(self, fs): return self._op("fftcosine", fs)
    def central_diffz(self, fs): return self._op("central_diffz", fs)
    def decompose_semi_spectral(self, sf): return self._op("decompose_semi_spectral", sf)
    def combine_semi_spectral(self, sf): return self._op("combine_semi_spectral", sf)
    def decompose_physical(self, fc): return self._op("decompose_physical", fc)
    def combine_physical(self, sf): return self._op("combine_physical", sf)
    def diffz(self, fs): return self._op("diffz", fs)

    # -------------------------------------------------------------- state
    def _fshape(self, name):
        return self.shape if name in SCALAR_FIELDS else (3,) + self.shape

    def get(self, name):
        out = np.zeros(self._fshape(name))
        self._chk(self.L.ps3d_gpu_get_field(self._h, FIELDS[name], _ptr(out)))
        return out

    def set(self, name, a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        assert a.shape == self._fshape(name)
        self._chk(self.L.ps3d_gpu_set_field(self._h, FIELDS[name], _ptr(a)))

    def table(self, name):
        w = TABLES[name]
        n2 = self.nx * self.ny
        n = {0: n2, 1: n2, 12: n2, 18: n2, 10: self.nz + 1, 11: self.nz + 1, 13: self.nx,
             14: self.ny, 15: self.nz + 1, 19: self.nz + 1}.get(w, n2 * (self.nz + 1))
        out = np.zeros(n)
        self._chk(self.L.ps3d_gpu_get_table(self._h, w, _ptr(out)))
        if n == n2 * (self.nz + 1):
            return out.reshape(self.shape)
        if n == n2 and w in (0, 1, 12, 18):
            return out.reshape(self.nx, self.ny)
        return out

    @property
    def ini_vor_mean(self):
        o = np.zeros(2)
        self._chk(self.L.ps3d_gpu_get_ini_vor_mean(self._h, _ptr(o)))
        return o

    @ini_vor_mean.setter
    def ini_vor_mean(self, v):
        v = np.ascontiguousarray(v, dtype=np.float64)
        self._chk(self.L.ps3d_gpu_set_ini_vor_mean(self._h, _ptr(v)))

    # ------------------------------------------------- reference routines
    def setup_fields(self, vor_phys, pert=None, buoy=None):
        """setup_fields (utils.f90:136-184); buoy is the total physical
        buoyancy of a buoyancy context (zero when omitted)."""
        vor_phys = np.ascontiguousarray(vor_phys, dtype=np.float64)
        assert vor_phys.shape == (3,) + self.shape
        pp = None
        if pert is not None:
            pert = np.ascontiguousarray(pert, dtype=np.float64)
            assert pert.shape == (3,) + self.shape
            pp = _ptr(pert)
        te, en = ctypes.c_double(), ctypes.c_double()
        if self.cfg.buoyancy:
            buoy = np.zeros(self.shape) if buoy is None else np.ascontiguousarray(buoy, dtype=np.float64)
            assert buoy.shape == self.shape
            self._chk(self.L.ps3d_gpu_setup_fields_buoyancy(self._h, _ptr(vor_phys), pp, _ptr(buoy),
                                                            ctypes.byref(te), ctypes.byref(en)))
        else:
            self._chk(self.L.ps3d_gpu_setup_fields(self._h, _ptr(vor_phys), pp, ctypes.byref(te),
                                                   ctypes.byref(en)))
        return te.value, en.value

    def buoyancy_params(self):
        """(N^2, buoyancy viscosity) of a buoyancy context."""
        b, v = ctypes.c_double(), ctypes.c_double()
        self._chk(self.L.ps3d_gpu_buoyancy_params(self._h, ctypes.byref(b), ctypes.byref(v)))
        return b.value, v.value

    def buoyancy_diagnostics(self):
        """(ape, gradb integral, min static stability, min Richardson number)"""
        out = np.zeros(4)
        self._chk(self.L.ps3d_gpu_buoyancy_diagnostics(self._h, _ptr(out)))
        return tuple(out)

    def set_diffusion_vb(self, dt, vpref, bpref):
        self._chk(self.L.ps3d_gpu_set_diffusion_vb(self._h, dt, vpref, bpref))

    def init_diffusion(self, te, en):
        self._chk(self.L.ps3d_gpu_init_diffusion(self._h, te, en))

    def vor2vel(self):
        self._chk(self.L.ps3d_gpu_vor2vel(self._h))

    def source(self):
        self._chk(self.L.ps3d_gpu_source(self._h))

    def adapt(self, t):
        dt = ctypes.c_double()
        d = _lib.Diag()
        self._chk(self.L.ps3d_gpu_adapt(self._h, t, ctypes.byref(dt), ctypes.byref(d)))
        return dt.value, d.as_dict()

    def set_diffusion(self, dt, pref):
        self._chk(self.L.ps3d_gpu_set_diffusion(self._h, dt, pref))

    def step(self, t, dt):
        tt = ctypes.c_double(t)
        self._chk(self.L.ps3d_gpu_step(self._h, ctypes.byref(tt), dt))
        return tt.value

    def advance(self, t):
        tt = ctypes.c_double(t)
        d = _lib.Diag()
        self._chk(self.L.ps3d_gpu_advance(self._h, ctypes.byref(tt), 1, ctypes.byref(d)))
        return tt.value, d.as_dict()

    def advance_n(self, t, nsteps):
        """nsteps advances; returns (t, list of per-step diagnostics)."""
        tt = ctypes.c_double(t)
        arr = (_lib.Diag * max(nsteps, 1))()
        self._chk(self.L.ps3d_gpu_advance(self._h, ctypes.byref(tt), nsteps, arr))
        return tt.value, [arr[i].as_dict() for i in range(nsteps)]

    def advance_host(self, svor, t):
        """One advance for a caller that owns svor on the host (in place)."""
        assert svor.dtype == np.float64 and svor.flags["C_CONTIGUOUS"]
        tt = ctypes.c_double(t)
        d = _lib.Diag()
        self._chk(self.L.ps3d_gpu_advance_host(self._h, _ptr(svor), ctypes.byref(tt), ctypes.byref(d)))
        return tt.value, d.as_dict()

    def time_advance(self, t, nsteps):
        """Device time (ms) of nsteps resident advances (CUDA events)."""
        tt = ctypes.c_double(t)
        ms = ctypes.c_double()
        self._chk(self.L.ps3d_gpu_time_advance(self._h, ctypes.byref(tt), nsteps, ctypes.byref(ms)))
        return tt.value, ms.value

    def derived_fields(self):
        """(pressure, horizontal divergence) of the current state, physical
        (nx, ny, nz+1) arrays (fields_derived.f90:67-182)."""
        shape = (self.nx, self.ny, self.nz + 1)
        p, dl = np.zeros(shape), np.zeros(shape)
        self._chk(self.L.ps3d_gpu_derived_fields(self._h, p.ctypes.data, dl.ctypes.data))
        return p, dl

    def ke_spectrum(self, nmax=8192):
        """(shell spectrum, dk) of the current vel (genspec.f90:42-123)."""
        spec = np.zeros(nmax)
        nb, dk = ctypes.c_int(), ctypes.c_double()
        self._chk(self.L.ps3d_gpu_ke_spectrum(self._h, nmax, _ptr(spec), ctypes.byref(nb), ctypes.byref(dk)))
        return spec[:nb.value], dk.value

    def tuning(self):
        """Line-FFT autotuner result: (shape per pass [fwd y, fwd x, inv y,
        inv x], ms per launch of shapes 0, 1, 2 per pass, 0 where a shape
        was not timed)."""
        sh = (ctypes.c_int * 4)()
        ms = (ctypes.c_double * 12)()
        self._chk(self.L.ps3d_gpu_tuning(self._h, sh, ms))
        return list(sh), [list(ms[3 * i:3 * i + 3]) for i in range(4)]

    def set_tuning(self, shapes):
        """Pin the line-FFT block shape per pass (-1 = default)."""
        self._chk(self.L.ps3d_gpu_set_tuning(self._h, (ctypes.c_int * 4)(*shapes)))

    def advance_graph(self, t, nsteps):
        """nsteps captured advances (mixed form, impl-diff-rk4): one CUDA graph
        launch per step, adapt's scalars on the device.  Returns (t, diag of
        the last step, device ms)."""
        tt = ctypes.c_double(t)
        ms = ctypes.c_double()
        d = _lib.Diag()
        self._chk(self.L.ps3d_gpu_advance_graph(self._h, ctypes.byref(tt), nsteps, ctypes.byref(d),
                                                ctypes.byref(ms)))
        return tt.value, d.as_dict(), ms.value

    def energy_series(self):
        a, b, c = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        self._chk(self.L.ps3d_gpu_energy_series(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
        return a.value, b.value, c.value

    def calc_vorticity_mean(self):
        o = np.zeros(2)
        self._chk(self.L.ps3d_gpu_calc_vorticity_mean(self._h, _ptr(o)))
        return o

    def adjust_vorticity_mean(self):
        self._chk(self.L.ps3d_gpu_adjust_vorticity_mean(self._h))

    def probe(self, kind):
        """Bracket launches of one kernel class with events (0 off, 1 y lines,
        2 x lines, 3 columns, 4 lines of both directions)."""
        self._chk(self.L.ps3d_gpu_probe(self._h, int(kind)))

    def probe_result(self):
        ms, n, b = ctypes.c_double(), ctypes.c_longlong(), ctypes.c_double()
        self._chk(self.L.ps3d_gpu_probe_result(self._h, ctypes.byref(ms), ctypes.byref(n), ctypes.byref(b)))
        return ms.value, n.value, b.value

    def save_state(self, path, t):
        """Checkpoint the run state at model time t (ps3d_gpu_save_state)."""
        self._chk(self.L.ps3d_gpu_save_state(self._h, str(path).encode(), float(t)))

    def load_state(self, path):
        """Restore a checkpoint of this configuration; returns its model time."""
        t = ctypes.c_double()
        self._chk(self.L.ps3d_gpu_load_state(self._h, str(path).encode(), ctypes.byref(t)))
        return t.value

    def synchronize(self):
        self._chk(self.L.ps3d_gpu_synchronize(self._h))


def batch_advance(models, ts, nsteps):
    """Advance independent runs (Ps3dGpu objects, any sizes, one device,
    mixed form, impl-diff-rk4) by nsteps steps, each step one CUDA graph for
    the whole batch: every run's right-hand sides on its own stream and one
    persistent launch per stage update for all runs (ps3d_gpu_batch_advance).
    Returns (list of times, device ms of the batch)."""
    n = len(models)
    hs = (ctypes.c_void_p * n)(*[m._h.value for m in models])
    tt = (ctypes.c_double * n)(*ts)
    ms = ctypes.c_double()
    L = models[0].L
    rc = L.ps3d_gpu_batch_advance(hs, n, tt, nsteps, ctypes.byref(ms))
    if rc:
        msgs = [L.ps3d_gpu_last_error(m._h).decode() for m in models]
        raise Ps3dError(rc, " | ".join(x for x in msgs if x))
    return list(tt), ms.value


class PinnedArray:
    """A page-locked FP64 host array from the library (ps3d_gpu_host_alloc);
    `.array` is the numpy view, valid until close()."""

    def __init__(self, shape):
        self.L = _lib.lib()
        n = int(np.prod(shape)) * 8
        self._p = ctypes.c_void_p()
        rc = self.L.ps3d_gpu_host_alloc(n, ctypes.byref(self._p))
        if rc:
            raise Ps3dError(rc, "ps3d_gpu_host_alloc")
        buf = (ctypes.c_double * (n // 8)).from_address(self._p.value)
        self.array = np.frombuffer(buf, dtype=np.float64).reshape(shape)

    def close(self):
        if self._p:
            self.array = None
            self.L.ps3d_gpu_host_free(self._p)
            self._p = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
