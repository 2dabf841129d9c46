"""ctypes binding of libps3d_gpu.so (the C ABI of include/ps3d_gpu.h).

Loading never falls back to anything: if the shared object is missing it is
built from csrc/ with nvcc, and if that fails the import error propagates.
"""
import ctypes
import os

from . import build as _build

_LIB = None
_dp = ctypes.POINTER(ctypes.c_double)
_vp = ctypes.c_void_p

OK = 0
ERRORS = {1: "INVALID_ARG", 2: "UNSUPPORTED_SIZE", 3: "CUDA", 4: "OUT_OF_MEMORY",
          5: "NOT_READY", 6: "NONFINITE", 7: "DEVICE_LIMIT", 8: "NO_DEVICE"}

# every entry point declared in include/ps3d_gpu.h
EXPORTS = [
    "ps3d_gpu_create", "ps3d_gpu_destroy", "ps3d_gpu_strerror", "ps3d_gpu_last_error",
    "ps3d_gpu_device_bytes", "ps3d_gpu_set_field", "ps3d_gpu_get_field",
    "ps3d_gpu_set_ini_vor_mean", "ps3d_gpu_get_ini_vor_mean", "ps3d_gpu_get_table",
    "ps3d_gpu_setup_fields", "ps3d_gpu_init_diffusion", "ps3d_gpu_vor2vel", "ps3d_gpu_source",
    "ps3d_gpu_adapt", "ps3d_gpu_set_diffusion", "ps3d_gpu_step", "ps3d_gpu_advance",
    "ps3d_gpu_advance_host", "ps3d_gpu_calc_vorticity_mean", "ps3d_gpu_adjust_vorticity_mean",
    "ps3d_gpu_energy_series", "ps3d_gpu_field_op", "ps3d_gpu_time_advance",
    "ps3d_gpu_launch_count", "ps3d_gpu_synchronize", "ps3d_gpu_probe", "ps3d_gpu_probe_result",
    "ps3d_gpu_energy_series_noalloc", "ps3d_gpu_advance_graph", "ps3d_gpu_batch_advance",
    "ps3d_gpu_tuning", "ps3d_gpu_set_tuning", "ps3d_gpu_derived_fields",
    "ps3d_gpu_ke_spectrum", "ps3d_gpu_host_alloc", "ps3d_gpu_host_free",
    "ps3d_gpu_setup_fields_buoyancy", "ps3d_gpu_buoyancy_params", "ps3d_gpu_set_diffusion_vb",
    "ps3d_gpu_buoyancy_diagnostics",
    "ps3d_closure_create", "ps3d_closure_destroy", "ps3d_closure_last_error",
    "ps3d_closure_get_params", "ps3d_closure_set_params", "ps3d_closure_get_scale",
    "ps3d_closure_set_scale", "ps3d_closure_add_sample", "ps3d_closure_num_samples",
    "ps3d_closure_train", "ps3d_closure_predict", "ps3d_closure_gradients", "ps3d_gpu_set_closure",
    "ps3d_closure_time_forward", "ps3d_closure_set_engine", "ps3d_closure_get_engine", "ps3d_closure_check",
    "ps3d_gpu_save_state", "ps3d_gpu_load_state",
]


class Config(ctypes.Structure):
    """ps3d_gpu_config (include/ps3d_gpu.h)."""

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
        ("precision", ctypes.c_int), ("device", ctypes.c_int),
        ("buoyancy", ctypes.c_int), ("bfsq", ctypes.c_double), ("bfsq_given", ctypes.c_int),
        ("buoy_nnu", ctypes.c_int), ("buoy_prediss", ctypes.c_double),
        ("buoy_pretype", ctypes.c_int), ("buoy_length_scale", ctypes.c_int),
        ("buoy_roll_mean_win_size", ctypes.c_int),
    ]


class Diag(ctypes.Structure):
    """ps3d_gpu_diag (include/ps3d_gpu.h)."""

    _fields_ = [(n, ctypes.c_double) for n in (
        "t", "dt", "ke", "en", "hel", "vortmax", "vortrms", "vorch")] + [
        ("vormean", ctypes.c_double * 3)] + [(n, ctypes.c_double) for n in (
            "ggmax", "usggmax", "lsggmax", "umax", "vmax", "wmax", "bfmax", "rmv", "pref",
            "rmb", "bpref")]

    def as_dict(self):
        d = {n: getattr(self, n) for n, _ in self._fields_ if n != "vormean"}
        d["vormean"] = list(self.vormean)
        return d


def path():
    return _build.LIB


def lib(build_if_missing=True):
    """Load libps3d_gpu.so; raises if it cannot be loaded."""
    global _LIB
    if _LIB is not None:
        return _LIB
    p = _build.LIB
    if build_if_missing and not _build.up_to_date():
        _build.build()
    if not os.path.exists(p):
        raise ImportError(f"{p} is missing: build it with ps3d_gb300.build.build()")
    L = ctypes.CDLL(p)
    L.ps3d_gpu_create.argtypes = [ctypes.POINTER(Config), ctypes.POINTER(_vp)]
    L.ps3d_gpu_destroy.argtypes = [_vp]
    L.ps3d_gpu_strerror.argtypes = [ctypes.c_int]
    L.ps3d_gpu_strerror.restype = ctypes.c_char_p
    L.ps3d_gpu_last_error.argtypes = [_vp]
    L.ps3d_gpu_last_error.restype = ctypes.c_char_p
    L.ps3d_gpu_device_bytes.argtypes = [_vp]
    L.ps3d_gpu_device_bytes.restype = ctypes.c_longlong
    L.ps3d_gpu_launch_count.argtypes = [_vp]
    L.ps3d_gpu_launch_count.restype = ctypes.c_longlong
    L.ps3d_gpu_set_field.argtypes = [_vp, ctypes.c_int, _dp]
    L.ps3d_gpu_get_field.argtypes = [_vp, ctypes.c_int, _dp]
    L.ps3d_gpu_set_ini_vor_mean.argtypes = [_vp, _dp]
    L.ps3d_gpu_get_ini_vor_mean.argtypes = [_vp, _dp]
    L.ps3d_gpu_get_table.argtypes = [_vp, ctypes.c_int, _dp]
    L.ps3d_gpu_setup_fields.argtypes = [_vp, _dp, _dp, _dp, _dp]
    L.ps3d_gpu_init_diffusion.argtypes = [_vp, ctypes.c_double, ctypes.c_double]
    L.ps3d_gpu_vor2vel.argtypes = [_vp]
    L.ps3d_gpu_source.argtypes = [_vp]
    L.ps3d_gpu_adapt.argtypes = [_vp, ctypes.c_double, _dp, ctypes.POINTER(Diag)]
    L.ps3d_gpu_set_diffusion.argtypes = [_vp, ctypes.c_double, ctypes.c_double]
    L.ps3d_gpu_set_diffusion_vb.argtypes = [_vp, ctypes.c_double, ctypes.c_double, ctypes.c_double]
    L.ps3d_gpu_setup_fields_buoyancy.argtypes = [_vp, _dp, _dp, _dp, _dp, _dp]
    L.ps3d_gpu_buoyancy_params.argtypes = [_vp, _dp, _dp]
    L.ps3d_gpu_buoyancy_diagnostics.argtypes = [_vp, _dp]
    L.ps3d_gpu_step.argtypes = [_vp, _dp, ctypes.c_double]
    L.ps3d_gpu_advance.argtypes = [_vp, _dp, ctypes.c_int, ctypes.POINTER(Diag)]
    L.ps3d_gpu_advance_host.argtypes = [_vp, _dp, _dp, ctypes.POINTER(Diag)]
    L.ps3d_gpu_calc_vorticity_mean.argtypes = [_vp, _dp]
    L.ps3d_gpu_adjust_vorticity_mean.argtypes = [_vp]
    L.ps3d_gpu_energy_series.argtypes = [_vp, _dp, _dp, _dp]
    L.ps3d_gpu_field_op.argtypes = [_vp, ctypes.c_int, _dp, _dp]
    L.ps3d_gpu_time_advance.argtypes = [_vp, _dp, ctypes.c_int, _dp]
    L.ps3d_gpu_tuning.argtypes = [_vp, ctypes.POINTER(ctypes.c_int), _dp]
    L.ps3d_gpu_derived_fields.argtypes = [_vp, ctypes.c_void_p, ctypes.c_void_p]
    L.ps3d_gpu_host_alloc.argtypes = [ctypes.c_size_t, ctypes.POINTER(ctypes.c_void_p)]
    L.ps3d_gpu_host_free.argtypes = [ctypes.c_void_p]
    L.ps3d_gpu_ke_spectrum.argtypes = [_vp, ctypes.c_int, _dp, ctypes.POINTER(ctypes.c_int), _dp]
    L.ps3d_gpu_set_tuning.argtypes = [_vp, ctypes.POINTER(ctypes.c_int)]
    L.ps3d_gpu_advance_graph.argtypes = [_vp, _dp, ctypes.c_int, ctypes.c_void_p, _dp]
    L.ps3d_gpu_batch_advance.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int, _dp, ctypes.c_int, _dp]
    L.ps3d_gpu_synchronize.argtypes = [_vp]
    L.ps3d_gpu_probe.argtypes = [_vp, ctypes.c_int]
    L.ps3d_gpu_probe_result.argtypes = [_vp, _dp, ctypes.POINTER(ctypes.c_longlong), _dp]
    L.ps3d_gpu_energy_series_noalloc.argtypes = [_vp, _vp, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                                 ctypes.c_longlong, ctypes.c_longlong, _vp, _vp]
    _fp = ctypes.POINTER(ctypes.c_float)
    L.ps3d_closure_create.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                      ctypes.c_ulonglong, ctypes.POINTER(_vp)]
    L.ps3d_closure_destroy.argtypes = [_vp]
    L.ps3d_closure_last_error.argtypes = [_vp]
    L.ps3d_closure_last_error.restype = ctypes.c_char_p
    L.ps3d_closure_get_params.argtypes = [_vp, _fp]
    L.ps3d_closure_set_params.argtypes = [_vp, _fp]
    L.ps3d_closure_get_scale.argtypes = [_vp, _dp]
    L.ps3d_closure_set_scale.argtypes = [_vp, ctypes.c_double]
    L.ps3d_closure_add_sample.argtypes = [_vp, _dp, _dp, _dp]
    L.ps3d_closure_num_samples.argtypes = [_vp, ctypes.POINTER(ctypes.c_int)]
    L.ps3d_closure_train.argtypes = [_vp, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_ulonglong, _dp]
    L.ps3d_closure_predict.argtypes = [_vp, _dp, _dp, _dp]
    L.ps3d_closure_gradients.argtypes = [_vp, ctypes.c_int, _fp, _fp, _dp]
    L.ps3d_gpu_set_closure.argtypes = [_vp, _vp, ctypes.c_int]
    L.ps3d_closure_time_forward.argtypes = [_vp, ctypes.c_int, _dp]
    L.ps3d_closure_set_engine.argtypes = [_vp, ctypes.c_int]
    L.ps3d_closure_get_engine.argtypes = [_vp, ctypes.POINTER(ctypes.c_int)]
    L.ps3d_closure_check.argtypes = [_vp]
    L.ps3d_gpu_save_state.argtypes = [_vp, ctypes.c_char_p, ctypes.c_double]
    L.ps3d_gpu_load_state.argtypes = [_vp, ctypes.c_char_p, _dp]
    _LIB = L
    return L
