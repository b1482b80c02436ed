"""ctypes binding of the C ABI in ``include/qew_gpu.h``.

Loads the in-tree ``_lib/libqew_gb300.so``. There is no fallback: if the
library is missing or cannot be loaded, every call raises.
"""
from __future__ import annotations

import ctypes as C
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
# QEW_GB300_VARIANT=bounds_check loads the bounds-checked build (_lib/bounds_check/)
_VARIANT = os.environ.get("QEW_GB300_VARIANT", "")
LIB_PATH = os.path.join(HERE, "_lib", *((_VARIANT,) if _VARIANT else ()), "libqew_gb300.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "qew_gpu.h")
HEADERS = [HEADER, os.path.join(os.path.dirname(HERE), "include", "qew_runs.h")]

D, I, U64, VP = C.c_double, C.c_int, C.c_uint64, C.c_void_p
PD = C.POINTER(C.c_double)

QEW_OK = 0
QEW_ERR_INVALID = 1
QEW_ERR_ODD_LENGTH = 2
QEW_ERR_CUDA = 3
QEW_ERR_NOMEM = 4
QEW_ERR_TIMEOUT = 5
QEW_ERR_UNSUPPORTED = 6

QEW_FIELD_BSPLINE, QEW_FIELD_ZERO, QEW_FIELD_CONST = 0, 1, 2
QEW_FIELD_HARMONIC, QEW_FIELD_WASHBOARD, QEW_FIELD_SINCOS = 3, 4, 5
QEW_STORE_FP64, QEW_STORE_FP32, QEW_STORE_FP32_EDGE, QEW_STORE_FP64_POLY = 1, 2, 4, 8
QEW_PREC_FP64, QEW_PREC_FP32_SPLIT, QEW_PREC_FP64_REFERENCE = 0, 1, 2
QEW_LBFGS_PLAIN, QEW_LBFGS_RESIDENT = 0, 1
QEW_NOALLOC_MAX_N = 1048576
QEW_RK_PLAIN, QEW_RK_RESIDENT = 0, 1
QEW_TUNE_GRADIENT_POLY, QEW_TUNE_GRADIENT_SPLIT, QEW_TUNE_RK_SEARCH = 0, 1, 2
QEW_TUNE_LANGEVIN_RUN = 3
QEW_REQ_STATIC, QEW_REQ_LANGEVIN, QEW_REQ_DEPINNING = 0, 1, 2


class qew_params(C.Structure):
    _fields_ = [("physical_size", D), ("line_tension", D), ("driving_force", D), ("model", I)]


class qew_lbfgs_params(C.Structure):
    _fields_ = [("m", I), ("ftol", D), ("max_iter", I), ("c1", D), ("ls_shrink", D),
                ("max_ls", I), ("curvature_eps", D), ("precondition", I), ("precond_shift", D),
                ("ls_fallback", I)]


class qew_lbfgs_result(C.Structure):
    _fields_ = [("iterations", I), ("max_force", D), ("converged", I),
                ("n_func_evals", C.c_long), ("n_curvature_skips", C.c_long),
                ("n_ls_restarts", C.c_long)]


class qew_rk_params(C.Structure):
    _fields_ = [("dstep", D), ("max_advance", D), ("root_tol", D), ("sweep_tol", D),
                ("runaway", D), ("max_sweeps", I)]


class qew_rk_result(C.Structure):
    _fields_ = [("blocked", I), ("runaway", I), ("sweeps", I), ("total_advance", D),
                ("mean_h", D)]


class qew_bisect_result(C.Structure):
    _fields_ = [("f_c", D), ("f_lo", D), ("f_hi", D), ("blocks", I), ("n_blocked", I),
                ("n_runaway", I), ("n_timeout", I), ("f_hi_verdict", I), ("sweeps", C.c_long)]


class qew_fire_params(C.Structure):
    _fields_ = [("dt_max", D), ("dt_init", D), ("ftol", D), ("max_iter", I), ("n_min", I),
                ("f_inc", D), ("f_dec", D), ("alpha_start", D), ("f_alpha", D)]


class qew_fire_result(C.Structure):
    _fields_ = [("iterations", I), ("max_force", D), ("converged", I)]


class qew_ensemble_line(C.Structure):
    _fields_ = [("field", VP), ("d_h", VP), ("n", I), ("p", qew_params), ("precond_shift", D)]


class qew_ensemble_params(C.Structure):
    _fields_ = [("lbfgs", qew_lbfgs_params), ("ftol_fp32", D), ("max_iter_fp32", I)]


class qew_request(C.Structure):
    _fields_ = [("kind", I), ("n", I), ("rows", I), ("xi", D), ("seed", U64), ("model", I),
                ("line_tension", D), ("driving_force", D), ("ftol", D), ("steps", I),
                ("temperature", D), ("dt", D), ("f_step", D), ("f_max", D),
                ("bisect_rtol", D), ("max_sweeps", I), ("max_advance", D), ("runaway", D),
                ("h_out", VP)]


class qew_response(C.Structure):
    _fields_ = [("id", U64), ("kind", I), ("status", I), ("t_submit", D), ("t_start", D),
                ("t_end", D), ("iterations", I), ("value", D), ("max_force", D),
                ("converged", I)]


class qew_static_config(C.Structure):
    _fields_ = [("model", I), ("amplitude", D), ("xi", D), ("Lx", D), ("Ly", D), ("nx", I),
                ("ny", I), ("driving_force", D), ("pinning_lengths_over_xi", PD),
                ("n_pinning_lengths", I), ("ftol", D), ("max_iter", I), ("lbfgs_m", I)]


class qew_static_profile(C.Structure):
    _fields_ = [("pinning_length_over_xi", D), ("line_tension", D), ("result", qew_lbfgs_result)]


class qew_dynamic_config(C.Structure):
    _fields_ = [("model", I), ("amplitude", D), ("xi", D), ("pinning_length_over_xi", D),
                ("driving_force", D), ("Lx", D), ("Ly", D), ("nx", I), ("ny", I), ("seed", U64),
                ("tau", D), ("tl_start", D), ("tl_end", D), ("total_time", D), ("dt", D),
                ("precision", I)]


class qew_dynamic_result(C.Structure):
    _fields_ = [("dt", D), ("total_time", D), ("line_tension", D), ("steps", C.c_longlong),
                ("snapshots", I)]


class qew_depinning_config(C.Structure):
    _fields_ = [("model", I), ("amplitude", D), ("xi", D), ("pinning_length_over_xi", D),
                ("Lx", D), ("Ly", D), ("nx", I), ("ny", I), ("f_step", D), ("f_max", D),
                ("rp", qew_rk_params), ("bisect_rtol", D), ("precision", I)]


class qew_depinning_step(C.Structure):
    _fields_ = [("f", D), ("result", qew_rk_result)]


class qew_depinning_result(C.Structure):
    _fields_ = [("line_tension", D), ("f_c_upper_bound", D), ("steps", I), ("f_c", D),
                ("f_c_lo", D), ("f_c_hi", D), ("bisect_blocks", I)]


SNAPSHOT_FN = C.CFUNCTYPE(None, VP, D, PD, I)
DEPINNING_FN = C.CFUNCTYPE(None, VP, C.POINTER(qew_depinning_step), PD, I)


class QewError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__("%s (status %d)" % (msg, status))
        self.status = status


_lib = None

# name -> (restype, argtypes)
_SIGS = {
    "qew_status_string": (C.c_char_p, [I]),
    "qew_ctx_create": (I, [I, C.POINTER(VP)]),
    "qew_ctx_destroy": (I, [VP]),
    "qew_ctx_set_stream": (I, [VP, VP]),
    "qew_ctx_synchronize": (I, [VP]),
    "qew_last_error": (C.c_char_p, [VP]),
    "qew_ctx_launch_count": (U64, [VP]),
    "qew_field_create_from_host": (I, [VP, PD, I, I, D, D, I, C.POINTER(VP)]),
    "qew_field_create_from_device": (I, [VP, VP, I, I, D, D, I, C.POINTER(VP)]),
    "qew_field_create_analytic": (I, [VP, I, D, D, D, C.POINTER(VP)]),
    "qew_field_create_generated": (I, [VP, I, I, D, D, D, D, D, U64, I, C.POINTER(VP)]),
    "qew_field_create_seeded": (I, [VP, I, I, D, D, D, D, D, U64, I, C.POINTER(VP)]),
    "qew_field_destroy": (I, [VP]),
    "qew_field_get_coefficients": (I, [VP, VP, PD]),
    "qew_field_sample": (I, [VP, VP, VP, VP, I, VP, VP, VP]),
    "qew_objective": (I, [VP, VP, VP, I, C.POINTER(qew_params), PD]),
    "qew_objective_trial": (I, [VP, VP, VP, VP, D, I, C.POINTER(qew_params), PD]),
    "qew_gradient": (I, [VP, VP, VP, I, C.POINTER(qew_params), VP]),
    "qew_gradient_prec": (I, [VP, VP, VP, I, C.POINTER(qew_params), I, VP]),
    "qew_gradient_batch": (I, [VP, VP, I, VP, I, C.POINTER(qew_params), I, VP]),
    "qew_measure_fp64_fma_rate": (I, [VP, I, PD, PD]),
    "qew_ctx_set_barrier_limits": (I, [VP, C.c_longlong, I]),
    "qew_ctx_set_autotune": (I, [VP, I]),
    "qew_bounds_check_report": (I, [C.POINTER(C.c_longlong)]),
    "qew_ctx_force_tune_candidate": (I, [VP, I, I]),
    "qew_tune_report": (I, [C.c_char_p, I]),
    "qew_gradient_host": (I, [VP, VP, VP, I, C.POINTER(qew_params), I, VP]),
    "qew_gradient_host_batch": (I, [VP, VP, I, VP, I, C.POINTER(qew_params), I, VP]),
    "qew_split_heights": (I, [VP, VP, VP, I, VP, VP]),
    "qew_join_heights": (I, [VP, VP, VP, VP, I, VP]),
    "qew_gradient_split": (I, [VP, VP, VP, VP, I, C.POINTER(qew_params), VP]),
    "qew_gradient_split_batch": (I, [VP, VP, I, VP, VP, I, C.POINTER(qew_params), VP]),
    "qew_objective_noalloc": (I, [VP, VP, I, C.POINTER(qew_params), VP, VP]),
    "qew_lbfgs_default_params": (I, [C.POINTER(qew_lbfgs_params)]),
    "qew_lbfgs_minimize": (I, [VP, VP, VP, I, C.POINTER(qew_params),
                               C.POINTER(qew_lbfgs_params), C.POINTER(qew_lbfgs_result)]),
    "qew_lbfgs_minimize_form": (I, [VP, VP, VP, I, C.POINTER(qew_params),
                                    C.POINTER(qew_lbfgs_params), I,
                                    C.POINTER(qew_lbfgs_result)]),
    "qew_precond_apply": (I, [VP, VP, I, D, D, D, I, VP]),
    "qew_ensemble_minimize": (I, [VP, I, C.POINTER(qew_ensemble_line),
                                  C.POINTER(qew_ensemble_params), C.POINTER(qew_lbfgs_result)]),
    "qew_server_create": (I, [I, D, I, C.POINTER(VP)]),
    "qew_server_submit": (I, [VP, C.POINTER(qew_request), C.POINTER(U64)]),
    "qew_server_lane_stats": (I, [VP, C.POINTER(U64), C.POINTER(U64)]),
    "qew_server_set_lane_limit": (I, [VP, I]),
    "qew_server_poll": (I, [VP, C.POINTER(qew_response), I]),
    "qew_server_drain": (I, [VP, D]),
    "qew_server_clock": (D, [VP]),
    "qew_server_destroy": (I, [VP]),
    "qew_langevin_create": (I, [VP, I, U64, C.POINTER(VP)]),
    "qew_langevin_destroy": (I, [VP]),
    "qew_langevin_step": (I, [VP, VP, VP, C.POINTER(qew_params), D, D]),
    "qew_langevin_step_increments": (I, [VP, VP, VP, C.POINTER(qew_params), D, D, VP]),
    "qew_langevin_peek_increments": (I, [VP, VP]),
    "qew_langevin_run": (I, [VP, VP, VP, C.POINTER(qew_params), I, PD, PD, I]),
    "qew_langevin_steps": (U64, [VP]),
    "qew_rk_site_velocity": (I, [VP, VP, VP, I, C.POINTER(qew_params), VP]),
    "qew_rk_block": (I, [VP, VP, VP, I, C.POINTER(qew_params), C.POINTER(qew_rk_params),
                         C.POINTER(qew_rk_result)]),
    "qew_depinning_bisect": (I, [VP, VP, VP, I, C.POINTER(qew_params),
                                 C.POINTER(qew_rk_params), D, D, D, I, PD, PD, PD,
                                 C.POINTER(I)]),
    "qew_rk_block_form": (I, [VP, VP, VP, I, C.POINTER(qew_params), C.POINTER(qew_rk_params),
                              I, I, C.POINTER(qew_rk_result)]),
    "qew_depinning_bisect_prec": (I, [VP, VP, VP, I, C.POINTER(qew_params),
                                      C.POINTER(qew_rk_params), D, D, D, I, I, PD, PD, PD,
                                      C.POINTER(I)]),
    "qew_depinning_bisect_ex": (I, [VP, VP, VP, I, C.POINTER(qew_params),
                                    C.POINTER(qew_rk_params), D, D, D, I, I,
                                    C.POINTER(qew_bisect_result), C.POINTER(I)]),
    "qew_fire_default_params": (I, [C.POINTER(qew_fire_params)]),
    "qew_fire_minimize": (I, [VP, VP, VP, I, C.POINTER(qew_params), C.POINTER(qew_fire_params),
                              C.POINTER(qew_fire_result)]),
    "qew_line_statistics": (I, [VP, I, VP, I, D, VP, VP, VP, VP]),
    "qew_line_statistics_host": (I, [VP, I, VP, I, D, VP, VP, VP, VP]),
    # drivers (qew_runs.h)
    "qew_static_config_default": (None, [C.POINTER(qew_static_config)]),
    "qew_static_sweep": (I, [VP, VP, C.POINTER(qew_static_config),
                             C.POINTER(qew_static_profile), PD]),
    "qew_dynamic_config_default": (None, [C.POINTER(qew_dynamic_config)]),
    "qew_dynamic_anneal": (I, [VP, VP, C.POINTER(qew_dynamic_config), SNAPSHOT_FN, VP,
                               C.POINTER(qew_dynamic_result)]),
    "qew_depinning_config_default": (None, [C.POINTER(qew_depinning_config)]),
    "qew_depinning_ramp": (I, [VP, VP, C.POINTER(qew_depinning_config), DEPINNING_FN, VP,
                               C.POINTER(qew_depinning_result)]),
}


def header_symbols() -> list[str]:
    """Every function the public headers declare."""
    txt = "".join(open(h).read() for h in HEADERS)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\*?\s*(qew_[a-z0-9_]+)\s*\(",
                                 txt, re.M)))


def load(path: str = LIB_PATH):
    """Load the CUDA library (raises if it is not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError("qew_gb300: CUDA library %s is not built; run "
                           "qew_gb300.build.build() (there is no CPU fallback)" % path)
    lib = C.CDLL(path)
    for name, (rt, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = rt
        fn.argtypes = args
    _lib = lib
    return lib


def check(status: int, ctx=None, what: str = "") -> None:
    if status == QEW_OK:
        return
    lib = load()
    msg = lib.qew_status_string(status).decode()
    if ctx is not None:
        detail = lib.qew_last_error(ctx).decode()
        if detail:
            msg = detail
    if what:
        msg = what + ": " + msg
    if status in (QEW_ERR_INVALID, QEW_ERR_ODD_LENGTH):
        raise ValueError(msg)
    raise QewError(status, msg)
