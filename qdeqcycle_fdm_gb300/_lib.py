"""ctypes loader of ``libqdeq_gb300.so`` (the C ABI in ``include/qdeq.h``).

There is no fallback: if the library is missing or no CUDA device is
present, calls raise.  The library is built in-tree by
``qdeqcycle_fdm_gb300.build.build()``.
"""
from __future__ import annotations

import ctypes as C
import os

from .build import LIB

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_fp = C.POINTER(C.c_float)

QD_OK, QD_ERR_ARG, QD_ERR_CUDA, QD_ERR_NOMEM, QD_ERR_NOT_CONVERGED, QD_ERR_NEWTON, QD_ERR_STATE = range(7)
QD_TOL_ABS, QD_TOL_REL = 0, 1
QD_PREC_FP64, QD_PREC_MIXED = 0, 1

# (name, restype, argtypes) of every entry point declared in include/qdeq.h
EXPORTS = [
    ("qd_version", C.c_char_p, []),
    ("qd_last_error", C.c_char_p, []),
    ("qd_default_options", None, [C.c_void_p]),
    ("qd_solver_create", C.c_int, [C.c_int, C.c_int, C.c_double, _dp, _dp, C.c_void_p,
                                   C.POINTER(C.c_void_p)]),
    ("qd_solver_create_mapped", C.c_int, [C.c_int, C.c_int, C.c_double, _dp, _dp, _dp, C.c_void_p,
                                          C.POINTER(C.c_void_p)]),
    ("qd_solver_destroy", C.c_int, [C.c_void_p]),
    ("qd_solver_set_options", C.c_int, [C.c_void_p, C.c_void_p]),
    ("qd_get_stats", C.c_int, [C.c_void_p, C.c_void_p]),
    ("qd_solver_stream", C.c_void_p, [C.c_void_p]),
    ("qd_set_medium", C.c_int, [C.c_int, C.c_int, _dp, _dp]),
    ("qd_upload_u", C.c_int, [C.c_void_p, _dp]),
    ("qd_download_u", C.c_int, [C.c_void_p, _dp]),
    ("qd_ode_solve", C.c_int, [C.c_void_p, _ip, _dp, _dp]),
    ("qd_ode_solve_host", C.c_int, [C.c_void_p, _dp, _ip, _dp]),
    ("qd_mg_smooth", C.c_int, [C.c_void_p, C.c_int]),
    ("qd_mg_vcycle", C.c_int, [C.c_void_p]),
    ("qd_mg_residual_norm", C.c_int, [C.c_void_p, _dp]),
    ("qd_mg_time_kernel", C.c_int, [C.c_void_p, C.c_int, C.c_int, _dp]),
    ("qd_convert_f64_to_f32", C.c_int, [_dp, _fp, C.c_int]),
    ("qd_split_f64", C.c_int, [_dp, _fp, _fp, C.c_int]),
    ("qd_residual_norm_noalloc", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int,
                                           C.c_int, C.c_double, C.c_void_p, _dp]),
    ("qd_fault_setup", C.c_int, [C.c_void_p, _dp, _dp, _dp, _dp, _dp, _dp, C.c_double,
                                 C.c_double, C.c_double, C.c_double]),
    ("qd_set_boundary", C.c_int, [C.c_void_p, _dp, C.c_double, C.c_double, C.c_double]),
    ("qd_eval_stress_on_fault", C.c_int, [C.c_void_p, _dp, _dp]),
    ("qd_nrsearch", C.c_int, [C.c_void_p, _dp, _dp, _dp, _ip]),
    ("qd_cal_dpsi", C.c_int, [C.c_void_p, _dp, _dp, _dp]),
    ("qd_rk43_start", C.c_int, [C.c_void_p, C.c_void_p, _dp, _dp]),
    ("qd_rk43_step", C.c_int, [C.c_void_p, C.c_int, _ip]),
    ("qd_rk43_resume", C.c_int, [C.c_void_p, C.c_void_p, _dp, _dp, C.c_double, C.c_double, C.c_double,
                                 C.c_double, C.c_int]),
    ("qd_probe_bounded_wait", C.c_int, [C.c_void_p, C.c_int]),
    ("qd_ensemble_step", C.c_int, [C.POINTER(C.c_void_p), C.c_int, C.c_int, _ip]),
    ("qd_rk43_get_state", C.c_int, [C.c_void_p, _dp, _dp, _dp, _dp, _dp]),
    ("qd_rk43_get_scalars", C.c_int, [C.c_void_p, _dp, _ip]),
    ("qd_rk43_set_state", C.c_int, [C.c_void_p, _dp, _dp, _dp, _dp, C.c_double, C.c_double,
                                    C.c_double, C.c_double, C.c_int]),
    ("qd_set_solution_history", C.c_int, [C.c_void_p, C.c_int]),
    ("qd_rk43_step_host", C.c_int, [C.c_void_p, C.c_int, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _ip, _ip]),
    ("qd_set_newton_start", C.c_int, [C.c_void_p, C.c_int]),
    ("qd_set_tail_sweeps", C.c_int, [C.c_void_p, C.c_int]),
    ("qd_set_smooth_correction", C.c_int, [C.c_void_p, C.c_double]),
    ("qd_autotune", C.c_int, [C.c_void_p, C.c_int, C.c_void_p]),
    ("qd_set_tiles", C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    ("qd_solution_history_fit", C.c_int, [C.c_void_p, _dp, _ip]),
    ("qd_load_initial_u", C.c_int, [C.c_char_p, C.c_int, C.c_int, _dp]),
    ("qd_save_initial_u", C.c_int, [C.c_char_p, C.c_int, C.c_int, _dp]),
    ("qd_snapshot", C.c_int, [C.c_void_p, C.c_char_p, C.c_int, C.c_int]),
    ("qd_snapshot_wait", C.c_int, [C.c_void_p]),
    ("qd_checkpoint_save", C.c_int, [C.c_void_p, C.c_char_p]),
    ("qd_checkpoint_load", C.c_int, [C.c_void_p, C.c_char_p]),
    # include/qdeq_unet.h
    ("qd_unet_create", C.c_int, [C.c_int, C.c_int, C.c_ulonglong, C.POINTER(C.c_void_p)]),
    ("qd_unet_destroy", None, [C.c_void_p]),
    ("qd_unet_num_params", C.c_longlong, [C.c_void_p]),
    ("qd_unet_get_params", C.c_int, [C.c_void_p, _fp]),
    ("qd_unet_set_params", C.c_int, [C.c_void_p, _fp]),
    ("qd_unet_forward_host", C.c_int, [C.c_void_p, _fp, _fp]),
    ("qd_unet_loss_grad_host", C.c_int, [C.c_void_p, _fp, _fp, _fp, _fp]),
    ("qd_unet_train_step_host", C.c_int, [C.c_void_p, _fp, _fp, C.c_float, _fp]),
    ("qd_solver_warm_start", C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_float]),
    ("qd_solver_warm_start_gate", C.c_int, [C.c_void_p, C.c_double]),
    ("qd_solver_warm_start_cost", C.c_int, [C.c_void_p, C.c_double]),
    ("qd_unet_stats", C.c_int, [C.c_void_p, C.POINTER(C.c_longlong), _fp]),
    ("qd_unet_time", C.c_int, [C.c_void_p, C.c_int, C.c_int, _dp, _dp]),
]


class MgOptions(C.Structure):
    _fields_ = [("n_levels", C.c_int), ("nu_pre", C.c_int), ("nu_post", C.c_int),
                ("nu_coarse", C.c_int), ("tol_mode", C.c_int), ("tol", C.c_double),
                ("max_cycles", C.c_int), ("precision", C.c_int), ("surface_prolong", C.c_int),
                ("coarse_solve", C.c_int)]


class Rk43Params(C.Structure):
    _fields_ = [("tmax", C.c_double), ("ini_dt", C.c_double), ("mindt", C.c_double),
                ("maxdt", C.c_double), ("totTol", C.c_double), ("maxNumSteps", C.c_int)]


class Stats(C.Structure):
    _fields_ = [("solves", C.c_longlong), ("vcycles", C.c_longlong), ("attempts", C.c_longlong),
                ("steps", C.c_longlong), ("newton_iters", C.c_longlong),
                ("kernel_launches", C.c_longlong), ("net_solves", C.c_longlong),
                ("net_cycles_needed", C.c_double), ("net_cycles_taken", C.c_double),
                ("smooth_corrections", C.c_longlong), ("net_armed_solves", C.c_longlong)]


class Tuning(C.Structure):
    _fields_ = [("nu_pre", C.c_int), ("nu_post", C.c_int), ("box_up", C.c_int), ("box_down", C.c_int),
                ("us_best", C.c_double), ("us_initial", C.c_double), ("cycles_best", C.c_int),
                ("cycles_initial", C.c_int), ("candidates", C.c_int), ("replayed", C.c_int)]


class QdError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"qdeq error {code}: {msg}")
        self.code = code


_lib = None


def load(path: str = LIB):
    """Load the library (no GPU needed to load it)."""
    global _lib
    if _lib is not None and path == LIB:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with qdeqcycle_fdm_gb300.build.build() "
                           "(there is no CPU fallback)")
    L = C.CDLL(path)
    for name, res, args in EXPORTS:
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    if path == LIB:
        _lib = L
    return L


def check(rc: int) -> int:
    if rc != QD_OK:
        raise QdError(rc, load().qd_last_error().decode(errors="replace"))
    return rc
