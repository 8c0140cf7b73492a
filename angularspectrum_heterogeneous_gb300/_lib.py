"""ctypes binding of ``libasgb300.so`` (the C ABI declared in include/asg_gb300.h).

The library is loaded from the package directory; a missing library or a
missing CUDA device raises immediately -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libasgb300.so")

ASG_OK = 0
ERRORS = {
    -1: "ASG_ERR_ARG", -2: "ASG_ERR_SHAPE", -3: "ASG_ERR_NAN", -4: "ASG_ERR_STABILITY",
    -5: "ASG_ERR_TIMEOUT", -6: "ASG_ERR_CUDA", -7: "ASG_ERR_STATE", -8: "ASG_ERR_NOMEM",
    -9: "ASG_ERR_SUBCYCLES",
}
FLUX_RUSANOV, FLUX_RUSANOV_TVD, FLUX_KT, FLUX_KT_MINMOD = 1, 2, 3, 4

EXPORTED = [
    "asg_plan_create", "asg_plan_destroy", "asg_set_step_operators", "asg_add_screen",
    "asg_add_source", "asg_run", "asg_get_outputs", "asg_last_run_ms", "asg_apply_operator",
    "asg_flux_columns", "asg_last_error", "asg_version", "asg_set_profiling",
    "asg_kernel_stats", "asg_flux_columns_device", "asg_get_tuning", "asg_set_tuning",
    "asg_autotune", "asg_set_graphs", "asg_batch_create", "asg_batch_destroy",
    "asg_batch_set_graphs", "asg_batch_run", "asg_batch_last_run_ms",
    "asg_net_param_count", "asg_net_create", "asg_net_destroy", "asg_net_set_params",
    "asg_net_get_params", "asg_net_forward", "asg_net_train_step", "asg_flux_columns_learned",
    "asg_net_set_output_scale", "asg_add_source_compact", "asg_debug_set_barrier_skew",
    "asg_flux_columns_device_clamped", "asg_set_learned", "asg_learned_stats",
]
KERNEL_KINDS = ["xy_A", "t_nonlin", "xy_B", "t_mid", "xy_C", "t_end", "other"]


class ASGError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class StabilityError(ASGError):
    """N dZ/dT max|p| exceeded stabilityThreshold.  The reference restarts from
    z=0 with a step that cannot fall below dZmin, i.e. it never terminates
    (angular_spectrum_solver.py:1420-1439); this is reported instead."""


class SubcycleCapError(ASGError):
    """Per-column KT sub-cycling: some column needed more sub-cycles than the
    cap and ran above its CFL target.  The run completed; the outputs exist
    but do not meet the requested CFL target."""


class Config(C.Structure):
    _fields_ = [
        ("nX", C.c_int), ("nY", C.c_int), ("nT", C.c_int),
        ("dX", C.c_double), ("dY", C.c_double), ("dT", C.c_double), ("c0", C.c_double),
        ("rho0", C.c_double), ("beta", C.c_double), ("f0", C.c_double),
        ("split_step", C.c_int), ("flux", C.c_int), ("boundary_layer", C.c_int),
        ("freq_weighted", C.c_int), ("super_absorbing", C.c_int),
        ("super_absorbing_strength", C.c_double), ("nonlinear_obliquity", C.c_int),
        ("stability_threshold", C.c_double), ("adaptive_filter_strength", C.c_double),
        ("kt_cfl_target", C.c_double),
        ("kt_max_subcycles", C.c_int), ("pax_x", C.c_int), ("pax_y", C.c_int),
    ]


_DP = C.POINTER(C.c_double)


class Tuning(C.Structure):
    _fields_ = [("t_cols_flux", C.c_int), ("t_cols_plain", C.c_int),
                ("t_cols_stats", C.c_int), ("xy_clusters", C.c_int),
                ("xy_clusters_closing", C.c_int), ("xy_sync", C.c_int),
                ("t_prefetch", C.c_int), ("xy_bulk", C.c_int), ("xy_rows", C.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class StepOps(C.Structure):
    _fields_ = [
        ("dz", C.c_double), ("kx", _DP), ("ky", _DP), ("kt", _DP),
        ("kfilt_start", C.c_double), ("kfilt_max", C.c_double),
        ("alpha", _DP), ("alpha_star", _DP),
        ("atten_obliquity", C.c_int), ("atten_clip_negative", C.c_int),
        ("abl_x", _DP), ("abl_y", _DP), ("abl_t", _DP),
        ("fw_exponent", _DP), ("fw_taper_x", _DP), ("fw_taper_y", _DP),
        ("sa_wx", _DP), ("sa_wy", _DP), ("beta_tvd", C.c_double),
    ]


STEP_CB = C.CFUNCTYPE(None, C.c_void_p, C.c_int, C.c_double, C.c_void_p)

_lib = None


def load(require_device: bool = True):
    """Load the library (once).  Raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(
            f"{LIB_PATH} is missing: build it with "
            "`python -m angularspectrum_heterogeneous_gb300.build` (there is no CPU fallback)")
    lib = C.CDLL(LIB_PATH)
    P = C.c_void_p
    F = C.POINTER(C.c_float)
    lib.asg_plan_create.argtypes = [C.POINTER(Config), C.POINTER(P)]
    lib.asg_plan_destroy.argtypes = [P]
    lib.asg_set_step_operators.argtypes = [P, C.c_int, C.POINTER(StepOps)]
    lib.asg_add_screen.argtypes = [P, C.c_double, F, F]
    lib.asg_add_source.argtypes = [P, C.c_double, F]
    lib.asg_add_source_compact.argtypes = [P, C.c_double, C.POINTER(C.c_int), C.c_int, F]
    lib.asg_run.argtypes = [P, F, C.c_double, C.c_double, STEP_CB, P, C.POINTER(C.c_int)]
    lib.asg_get_outputs.argtypes = [P, F, F, F, F, F, _DP, F]
    lib.asg_last_run_ms.argtypes = [P, _DP]
    lib.asg_apply_operator.argtypes = [P, C.c_int, F, C.c_int, _DP]
    lib.asg_flux_columns.argtypes = [F, F, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double,
                                     C.c_double, C.c_double, C.c_double, C.c_int]
    lib.asg_flux_columns_device.argtypes = [P, P, C.c_int, C.c_int, C.c_int, C.c_double,
                                            C.c_double, C.c_double, C.c_double, C.c_double,
                                            C.c_int, P]
    lib.asg_flux_columns_device_clamped.argtypes = [P, C.POINTER(C.c_uint), C.POINTER(C.c_uint)]
    lib.asg_set_learned.argtypes = [P, P, C.c_int, C.c_float]
    lib.asg_learned_stats.argtypes = [P, C.POINTER(C.c_long), C.POINTER(C.c_long)]
    lib.asg_get_tuning.argtypes = [P, C.POINTER(Tuning)]
    lib.asg_set_tuning.argtypes = [P, C.POINTER(Tuning)]
    lib.asg_debug_set_barrier_skew.argtypes = [P, C.c_int]
    lib.asg_autotune.argtypes = [P, F, C.c_double, C.c_int, C.POINTER(Tuning)]
    lib.asg_set_graphs.argtypes = [P, C.c_int]
    lib.asg_net_param_count.argtypes = []
    lib.asg_net_create.argtypes = [C.POINTER(P)]
    lib.asg_net_destroy.argtypes = [P]
    lib.asg_net_set_params.argtypes = [P, F, C.c_int]
    lib.asg_net_get_params.argtypes = [P, F, C.c_int]
    lib.asg_net_forward.argtypes = [P, P, P, C.c_int, C.c_int, P]
    lib.asg_net_train_step.argtypes = [P, P, P, P, C.c_int, C.c_int, C.c_float, _DP, F]
    lib.asg_net_set_output_scale.argtypes = [P, C.c_float]
    lib.asg_flux_columns_learned.argtypes = [P, P, P, C.c_int, C.c_int, C.c_int, C.c_double,
                                             C.c_double, C.c_double, C.c_double, C.c_int,
                                             C.c_int, C.c_float, C.POINTER(C.c_int), P]
    lib.asg_batch_create.argtypes = [C.POINTER(P), C.c_int, C.POINTER(P)]
    lib.asg_batch_destroy.argtypes = [P]
    lib.asg_batch_set_graphs.argtypes = [P, C.c_int]
    lib.asg_batch_run.argtypes = [P, C.POINTER(F), _DP, _DP, C.POINTER(C.c_int)]
    lib.asg_batch_last_run_ms.argtypes = [P, _DP]
    lib.asg_set_profiling.argtypes = [P, C.c_int]
    lib.asg_kernel_stats.argtypes = [P, _DP, C.POINTER(C.c_long), C.c_int]
    lib.asg_last_error.restype = C.c_char_p
    lib.asg_version.restype = C.c_char_p
    for name in EXPORTED:
        if name not in ("asg_last_error", "asg_version"):
            getattr(lib, name).restype = C.c_int
    _lib = lib
    return lib


def check(code):
    if code == ASG_OK:
        return
    msg = _lib.asg_last_error().decode(errors="replace") if _lib is not None else ""
    if code == -4:
        raise StabilityError(code, msg)
    if code == -9:
        raise SubcycleCapError(code, msg)
    raise ASGError(code, msg)


def fptr(a: np.ndarray | None):
    if a is None:
        return None
    assert a.dtype == np.float32 and a.flags.c_contiguous
    return a.ctypes.data_as(C.POINTER(C.c_float))


def dptr(a: np.ndarray | None):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_DP)


def flux_columns(cols: np.ndarray, flux: int, n_coef: float, dz: float, dt: float,
                 beta_tvd: float = 1.0, cfl_target: float = 0.0, max_subcycles: int = 1024):
    """Burgers step on independent columns (last axis t) on the GPU."""
    lib = load()
    a = np.ascontiguousarray(cols, dtype=np.float32)
    nT = a.shape[-1]
    ncols = a.size // nT
    out = np.empty_like(a)
    check(lib.asg_flux_columns(fptr(a), fptr(out), ncols, nT, flux, n_coef, dz, dt, beta_tvd,
                               cfl_target, max_subcycles))
    return out
