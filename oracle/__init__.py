"""ctypes bindings for the CPU oracle (TEST INFRASTRUCTURE ONLY).

The oracle is a plain-C FP64 restatement of the reference Fortran hot path
(matt-frey/ps3d).  Only the tests, the smoke entry point and the benchmark's
CPU-baseline leg use it, to check results and to time the CPU; the GPU
product path never calls it.
Parity pinning: see tests/test_oracle_kat.py (the reference's own known-answer
unit tests, ported).
"""
import ctypes
import os

import numpy as np

from . import build as _build

_LIB = None


class Config(ctypes.Structure):
    """Mirror of ps3o_config (oracle/ps3d_oracle.h)."""

    _fields_ = [
        ("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
        ("nnu", ctypes.c_int),
        ("lower", ctypes.c_double * 3), ("extent", ctypes.c_double * 3),
        ("prediss", ctypes.c_double),
        ("pretype", ctypes.c_int), ("length_scale", ctypes.c_int),
        ("filtering", ctypes.c_int), ("stepper", ctypes.c_int),
        ("cflmax", ctypes.c_double), ("alpha", ctypes.c_double),
        ("time_limit", ctypes.c_double),
        ("roll_mean_win_size", ctypes.c_int), ("nthreads", ctypes.c_int),
        ("hold_source", ctypes.c_int),
        ("f_cor", ctypes.c_double * 3),
        ("buoyancy", ctypes.c_int), ("bfsq", ctypes.c_double), ("bfsq_given", ctypes.c_int),
        ("buoy_nnu", ctypes.c_int), ("buoy_prediss", ctypes.c_double),
        ("buoy_pretype", ctypes.c_int), ("buoy_length_scale", ctypes.c_int),
        ("buoy_roll_mean_win_size", ctypes.c_int),
    ]


class Diag(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in (
        "t", "dt", "ke", "en", "hel", "vortmax", "vortrms", "vorch")] + [
        ("vormean", ctypes.c_double * 3)] + [(n, ctypes.c_double) for n in (
            "ggmax", "usggmax", "lsggmax", "umax", "vmax", "wmax", "bfmax", "rmv", "pref",
            "rmb", "bpref")]

    def as_dict(self):
        d = {n: getattr(self, n) for n, _ in self._fields_ if n != "vormean"}
        d["vormean"] = list(self.vormean)
        return d


PRETYPES = {"constant": 0, "vorch": 1, "bfmax": 2, "roll-mean-max-strain": 3,
            "max-strain": 4, "us-max-strain": 5, "roll-mean-bfmax": 6}
LENGTH_SCALES = {"Kolmogorov": 0, "geophysical": 1}
FILTERS = {"Hou & Li": 0, "2/3-rule": 1}
STEPPERS = {"impl-diff-rk4": 0, "cn2": 1}
TABLES = {"k2l2": 0, "k2l2i": 1, "filt": 2, "green": 3, "phim": 4, "phip": 5,
          "thetam": 6, "thetap": 7, "dthetam": 8, "dthetap": 9, "gamtop": 10,
          "gambot": 11, "vhdis": 12, "rkx": 13, "rky": 14, "rkz": 15,
          "dphim": 16, "dphip": 17, "bhdis": 18, "bbarz": 19}
FIELDS = {"svor": 0, "vor": 1, "vel": 2, "svel": 3, "svorts": 4,
          "sbuoy": 5, "buoy": 6, "sbuoys": 7}
SCALAR_FIELDS = ("sbuoy", "buoy", "sbuoys")

_dp = ctypes.POINTER(ctypes.c_double)


def lib():
    global _LIB
    if _LIB is None:
        path = _build.build()
        L = ctypes.CDLL(path)
        vp = ctypes.c_void_p
        L.ps3o_create.argtypes = [ctypes.POINTER(Config), ctypes.POINTER(vp)]
        L.ps3o_destroy.argtypes = [vp]
        for name in ("ps3o_fftxyp2s", "ps3o_fftxys2p", "ps3o_diffx", "ps3o_diffy",
                     "ps3o_central_diffz", "ps3o_decompose_physical",
                     "ps3o_combine_physical"):
            getattr(L, name).argtypes = [vp, _dp, _dp]
        for name in ("ps3o_fftsine", "ps3o_fftcosine", "ps3o_decompose_semi_spectral",
                     "ps3o_combine_semi_spectral"):
            getattr(L, name).argtypes = [vp, _dp]
        L.ps3o_get_table.argtypes = [vp, ctypes.c_int, _dp]
        L.ps3o_get_field.argtypes = [vp, ctypes.c_int, _dp]
        L.ps3o_set_field.argtypes = [vp, ctypes.c_int, _dp]
        L.ps3o_get_ini_vor_mean.argtypes = [vp, _dp]
        L.ps3o_set_ini_vor_mean.argtypes = [vp, _dp]
        L.ps3o_get_vvisc.argtypes = [vp]
        L.ps3o_get_vvisc.restype = ctypes.c_double
        L.ps3o_setup_fields.argtypes = [vp, _dp, _dp, _dp, _dp]
        L.ps3o_init_diffusion.argtypes = [vp, ctypes.c_double, ctypes.c_double]
        L.ps3o_vor2vel.argtypes = [vp]
        L.ps3o_source.argtypes = [vp]
        L.ps3o_adapt.argtypes = [vp, ctypes.c_double, _dp, ctypes.POINTER(Diag)]
        L.ps3o_step.argtypes = [vp, _dp, ctypes.c_double]
        L.ps3o_set_diffusion.argtypes = [vp, ctypes.c_double, ctypes.c_double]
        L.ps3o_advance.argtypes = [vp, _dp, ctypes.POINTER(Diag)]
        L.ps3o_energy_series.argtypes = [vp, _dp, _dp, _dp]
        L.ps3o_calc_vorticity_mean.argtypes = [vp, _dp]
        L.ps3o_adjust_vorticity_mean.argtypes = [vp]
        L.ps3o_rolling_mean_next.argtypes = [vp, ctypes.c_double]
        L.ps3o_rolling_mean_next.restype = ctypes.c_double
        L.ps3o_jacobi_eigenvalues.argtypes = [_dp, _dp]
        L.ps3o_pressure.argtypes = [vp, _dp]
        L.ps3o_horizontal_divergence.argtypes = [vp, _dp]
        L.ps3o_ke_spectrum.argtypes = [vp, ctypes.c_int, _dp, _dp]
        L.ps3o_setup_fields_buoyancy.argtypes = [vp, _dp, _dp, _dp, _dp, _dp]
        L.ps3o_get_bfsq.argtypes = [vp]
        L.ps3o_get_bfsq.restype = ctypes.c_double
        L.ps3o_get_bvisc.argtypes = [vp]
        L.ps3o_get_bvisc.restype = ctypes.c_double
        L.ps3o_diffz.argtypes = [vp, _dp, _dp]
        L.ps3o_buoyancy_tendency.argtypes = [vp]
        L.ps3o_buoyancy_diagnostics.argtypes = [vp, _dp]
        L.ps3o_set_diffusion_vb.argtypes = [vp, ctypes.c_double, ctypes.c_double, ctypes.c_double]
        L.ps3o_forfft.argtypes = [ctypes.c_int, ctypes.c_int, _dp, _dp, _dp, ctypes.POINTER(ctypes.c_int)]
        L.ps3o_revfft.argtypes = L.ps3o_forfft.argtypes
        L.ps3o_dct.argtypes = [ctypes.c_int, ctypes.c_int, _dp, _dp, _dp, _dp, ctypes.POINTER(ctypes.c_int)]
        L.ps3o_dst.argtypes = L.ps3o_dct.argtypes
        L.ps3o_initfft.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_int), _dp]
        _LIB = L
    return _LIB


def _ptr(a):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_dp)


def make_config(nx, ny, nz, lower, extent, nnu=3, prediss=30.0, pretype="vorch",
                length_scale="Kolmogorov", filtering="Hou & Li",
                stepper="impl-diff-rk4", cflmax=0.8, alpha=0.1, time_limit=1.0e30,
                roll_mean_win_size=1000, nthreads=0, hold_source=0,
                f_cor=(0.0, 0.0, 0.0), buoyancy=False, bfsq=None, buoy_nnu=3,
                buoy_prediss=30.0, buoy_pretype="bfmax", buoy_length_scale="Kolmogorov",
                buoy_roll_mean_win_size=1000):
    c = Config()
    c.nx, c.ny, c.nz, c.nnu = nx, ny, nz, nnu
    c.lower[:] = list(lower)
    c.extent[:] = list(extent)
    c.prediss = prediss
    c.pretype = PRETYPES[pretype] if isinstance(pretype, str) else int(pretype)
    c.length_scale = LENGTH_SCALES[length_scale] if isinstance(length_scale, str) else int(length_scale)
    c.filtering = FILTERS[filtering] if isinstance(filtering, str) else int(filtering)
    c.stepper = STEPPERS[stepper] if isinstance(stepper, str) else int(stepper)
    c.cflmax, c.alpha, c.time_limit = cflmax, alpha, time_limit
    c.roll_mean_win_size, c.nthreads = roll_mean_win_size, nthreads
    c.hold_source = int(hold_source)
    c.f_cor[:] = list(f_cor)
    c.buoyancy = int(bool(buoyancy))
    c.bfsq = 0.0 if bfsq is None else float(bfsq)
    c.bfsq_given = int(bfsq is not None)
    c.buoy_nnu, c.buoy_prediss = buoy_nnu, buoy_prediss
    c.buoy_pretype = PRETYPES[buoy_pretype] if isinstance(buoy_pretype, str) else int(buoy_pretype)
    c.buoy_length_scale = (LENGTH_SCALES[buoy_length_scale] if isinstance(buoy_length_scale, str)
                           else int(buoy_length_scale))
    c.buoy_roll_mean_win_size = buoy_roll_mean_win_size
    return c


def _transform1d(fn, m, n, x):
    L = lib()
    x = np.ascontiguousarray(x, dtype=np.float64).copy()
    fac = (ctypes.c_int * 5)()
    trig = np.zeros(2 * n)
    if L.ps3o_initfft(n, fac, _ptr(trig)) != 0:
        raise ValueError(f"length {n} does not factorise into 2,3,4,5,6")
    wk = np.zeros(max(m * n, 1))
    if fn in ("dct", "dst"):
        wk2 = np.zeros(max(m * n, 1))
        getattr(L, "ps3o_" + fn)(m, n, _ptr(x), _ptr(wk), _ptr(wk2), _ptr(trig), fac)
    else:
        getattr(L, "ps3o_" + fn)(m, n, _ptr(x), _ptr(wk), _ptr(trig), fac)
    return x


def forfft(x):
    """Forward real FFT of a 1-D array (Hermitian storage, 1/sqrt(n))."""
    return _transform1d("forfft", 1, len(x), x)


def revfft(x):
    return _transform1d("revfft", 1, len(x), x)


def dct(x):
    """Self-inverse DCT of x[0..n] (len n+1)."""
    return _transform1d("dct", 1, len(x) - 1, x)


def dst(x):
    """Self-inverse DST of x[1..n] given as an array of length n (last := 0)."""
    return _transform1d("dst", 1, len(x), x)


def jacobi_eigenvalues(a):
    a = np.asfortranarray(np.array(a, dtype=np.float64)).ravel(order="F").copy()
    e = np.zeros(3)
    lib().ps3o_jacobi_eigenvalues(_ptr(a), _ptr(e))
    return e


class Oracle:
    """One FP64 CPU model of the reference hot path (single rank).

    Fields are numpy arrays shaped (3, nx, ny, nz+1) for vector fields and
    (nx, ny, nz+1) for scalars: C order of that shape is exactly the
    reference's Fortran (0:nz, 0:ny-1, 0:nx-1) column-major layout.
    """

    def __init__(self, nx, ny, nz, lower, extent, **kw):
        self.nx, self.ny, self.nz = nx, ny, nz
        self.cfg = make_config(nx, ny, nz, lower, extent, **kw)
        self._h = ctypes.c_void_p()
        rc = lib().ps3o_create(ctypes.byref(self.cfg), ctypes.byref(self._h))
        if rc != 0:
            raise ValueError(f"ps3o_create failed ({rc})")

    def close(self):
        if self._h:
            lib().ps3o_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def shape(self):
        return (self.nx, self.ny, self.nz + 1)

    def _s(self, a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        assert a.shape == self.shape, (a.shape, self.shape)
        return a

    def _call2(self, name, a):
        a = self._s(a)
        out = np.zeros(self.shape)
        getattr(lib(), name)(self._h, _ptr(a), _ptr(out))
        return out

    def _call1(self, name, a):
        a = self._s(a).copy()
        getattr(lib(), name)(self._h, _ptr(a))
        return a

    def fftxyp2s(self, fp): return self._call2("ps3o_fftxyp2s", fp)
    def fftxys2p(self, fs): return self._call2("ps3o_fftxys2p", fs)
    def diffx(self, fs): return self._call2("ps3o_diffx", fs)
    def diffy(self, fs): return self._call2("ps3o_diffy", fs)
    def central_diffz(self, fs): return self._call2("ps3o_central_diffz", fs)
    def decompose_physical(self, fc): return self._call2("ps3o_decompose_physical", fc)
    def combine_physical(self, sf): return self._call2("ps3o_combine_physical", sf)
    def fftsine(self, fs): return self._call1("ps3o_fftsine", fs)
    def fftcosine(self, fs): return self._call1("ps3o_fftcosine", fs)
    def decompose_semi_spectral(self, sf): return self._call1("ps3o_decompose_semi_spectral", sf)
    def combine_semi_spectral(self, sf): return self._call1("ps3o_combine_semi_spectral", sf)

    def table(self, name):
        w = TABLES[name]
        n = {0: self.nx * self.ny, 1: self.nx * self.ny, 12: self.nx * self.ny,
             10: self.nz + 1, 11: self.nz + 1, 13: self.nx, 14: self.ny,
             15: self.nz + 1, 18: self.nx * self.ny,
             19: self.nz + 1}.get(w, self.nx * self.ny * (self.nz + 1))
        out = np.zeros(n)
        if lib().ps3o_get_table(self._h, w, _ptr(out)) != 0:
            raise ValueError(f"table {name} not available")
        if n == self.nx * self.ny * (self.nz + 1):
            return out.reshape(self.shape)
        if n == self.nx * self.ny:
            return out.reshape(self.nx, self.ny)
        return out

    def _fshape(self, name):
        return self.shape if name in SCALAR_FIELDS else (3,) + self.shape

    def get(self, name):
        out = np.zeros(self._fshape(name))
        if lib().ps3o_get_field(self._h, FIELDS[name], _ptr(out)) != 0:
            raise ValueError(f"field {name} not available")
        return out

    def set(self, name, a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        assert a.shape == self._fshape(name)
        if lib().ps3o_set_field(self._h, FIELDS[name], _ptr(a)) != 0:
            raise ValueError(f"field {name} not available")

    @property
    def ini_vor_mean(self):
        o = np.zeros(2)
        lib().ps3o_get_ini_vor_mean(self._h, _ptr(o))
        return o

    @ini_vor_mean.setter
    def ini_vor_mean(self, v):
        v = np.ascontiguousarray(v, dtype=np.float64)
        lib().ps3o_set_ini_vor_mean(self._h, _ptr(v))

    @property
    def vvisc(self):
        return lib().ps3o_get_vvisc(self._h)

    def setup_fields(self, vor_phys, pert=None, buoy=None):
        """setup_fields; buoy is the total physical buoyancy (buoyancy runs)."""
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
            lib().ps3o_setup_fields_buoyancy(self._h, _ptr(vor_phys), pp, _ptr(buoy), ctypes.byref(te),
                                             ctypes.byref(en))
        else:
            lib().ps3o_setup_fields(self._h, _ptr(vor_phys), pp, ctypes.byref(te), ctypes.byref(en))
        return te.value, en.value

    @property
    def bfsq(self):
        return lib().ps3o_get_bfsq(self._h)

    @property
    def bvisc(self):
        return lib().ps3o_get_bvisc(self._h)

    def diffz(self, fs):
        fs = self._s(fs)
        out = np.zeros(self.shape)
        if lib().ps3o_diffz(self._h, _ptr(fs), _ptr(out)) != 0:
            raise ValueError("diffz needs a model built with buoyancy")
        return out
    def buoyancy_tendency(self): lib().ps3o_buoyancy_tendency(self._h)

    def buoyancy_diagnostics(self):
        """(ape, gradb integral, min static stability, min Richardson number)"""
        out = np.zeros(4)
        lib().ps3o_buoyancy_diagnostics(self._h, _ptr(out))
        return tuple(out)

    def set_diffusion_vb(self, dt, vpref, bpref):
        lib().ps3o_set_diffusion_vb(self._h, dt, vpref, bpref)

    def init_diffusion(self, te, en):
        lib().ps3o_init_diffusion(self._h, te, en)

    def vor2vel(self): lib().ps3o_vor2vel(self._h)
    def source(self): lib().ps3o_source(self._h)

    def adapt(self, t):
        dt = ctypes.c_double()
        d = Diag()
        lib().ps3o_adapt(self._h, t, ctypes.byref(dt), ctypes.byref(d))
        return dt.value, d.as_dict()

    def step(self, t, dt):
        tt = ctypes.c_double(t)
        lib().ps3o_step(self._h, ctypes.byref(tt), dt)
        return tt.value

    def set_diffusion(self, dt, pref):
        lib().ps3o_set_diffusion(self._h, dt, pref)

    def advance(self, t):
        tt = ctypes.c_double(t)
        d = Diag()
        lib().ps3o_advance(self._h, ctypes.byref(tt), ctypes.byref(d))
        return tt.value, d.as_dict()

    def pressure(self):
        out = np.zeros(self.shape)
        lib().ps3o_pressure(self._h, _ptr(out))
        return out

    def horizontal_divergence(self):
        out = np.zeros(self.shape)
        lib().ps3o_horizontal_divergence(self._h, _ptr(out))
        return out

    def ke_spectrum(self, nmax=4096):
        spec = np.zeros(nmax)
        dk = ctypes.c_double()
        nb = lib().ps3o_ke_spectrum(self._h, nmax, _ptr(spec), ctypes.byref(dk))
        return spec[:nb], dk.value

    def energy_series(self):
        a, b, c = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        lib().ps3o_energy_series(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c))
        return a.value, b.value, c.value

    def calc_vorticity_mean(self):
        o = np.zeros(2)
        lib().ps3o_calc_vorticity_mean(self._h, _ptr(o))
        return o

    def adjust_vorticity_mean(self):
        lib().ps3o_adjust_vorticity_mean(self._h)

    def rolling_mean_next(self, v):
        return lib().ps3o_rolling_mean_next(self._h, v)
