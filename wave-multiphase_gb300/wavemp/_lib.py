"""ctypes binding of libwavemp.so (include/wavemp.h). Raises if the library is missing."""
from __future__ import annotations

import ctypes
import os

from . import _build

WM_OK = 0
WM_ERR = {-1: "invalid argument", -2: "CUDA error", -3: "out of memory / workspace too small",
          -4: "call out of order"}

VARIANT = {"sc": 0, "m10": 1}
RECON = {"shipped": 0, "mp5c6": 1}
BC = {"transmissive": 0, "slip": 1, "reflective": 1}
PRECISION = {"fp64": 0, "fp32": 1}

WS_FX, WS_GY, WS_FXL, WS_GYL, WS_THETA, WS_SIGMA_X, WS_SIGMA_Y = 0, 7, 14, 21, 28, 31, 32


class WmParams(ctypes.Structure):
    _fields_ = [("gamma1", ctypes.c_double), ("pinf1", ctypes.c_double),
                ("gamma2", ctypes.c_double), ("pinf2", ctypes.c_double),
                ("dx", ctypes.c_double), ("dy", ctypes.c_double), ("cfl", ctypes.c_double),
                ("variant", ctypes.c_int), ("recon", ctypes.c_int), ("bc", ctypes.c_int * 4),
                ("emergency_repair", ctypes.c_int), ("precision", ctypes.c_int),
                ("fp64_switches", ctypes.c_int)]


class WmFields(ctypes.Structure):
    _fields_ = [(n, ctypes.c_void_p) for n in
                ("ar1", "ar2", "ru", "rv", "E", "al", "u_p", "v_p", "p_p", "al_prim")] + \
               [("pitch", ctypes.c_longlong)]


MAX_SAVES = 32


class WmSchedule(ctypes.Structure):
    _fields_ = [("t", ctypes.c_double), ("t_end", ctypes.c_double), ("step", ctypes.c_longlong),
                ("nsaves", ctypes.c_int), ("hit", ctypes.c_int), ("finished", ctypes.c_int),
                ("dt", ctypes.c_double), ("save_times", ctypes.c_double * MAX_SAVES),
                ("saved", ctypes.c_int * MAX_SAVES)]


class WmBatchParams(ctypes.Structure):
    _fields_ = [("variant", ctypes.c_int), ("recon", ctypes.c_int), ("precision", ctypes.c_int),
                ("emergency_repair", ctypes.c_int), ("g", ctypes.c_int), ("cfl", ctypes.c_double),
                ("tile_shape", ctypes.c_int), ("fp64_switches", ctypes.c_int),
                ("spin_limit", ctypes.c_longlong)]


class WmSolveDesc(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("dx", ctypes.c_double),
                ("dy", ctypes.c_double), ("gamma1", ctypes.c_double), ("pinf1", ctypes.c_double),
                ("gamma2", ctypes.c_double), ("pinf2", ctypes.c_double), ("bc", ctypes.c_int * 4),
                ("t_end", ctypes.c_double), ("max_steps", ctypes.c_longlong),
                ("q", WmFields), ("q_old", WmFields)]


class WmSolveStatus(ctypes.Structure):
    _fields_ = [("used", ctypes.c_int), ("done", ctypes.c_int), ("t", ctypes.c_double),
                ("dt", ctypes.c_double), ("steps", ctypes.c_longlong)]


class WmStats(ctypes.Structure):
    _fields_ = [("repaired_cells", ctypes.c_longlong), ("nonfinite_cells", ctypes.c_longlong),
                ("limited_cells", ctypes.c_longlong), ("steps", ctypes.c_longlong)]


EXPORTS = ("wm_version", "wm_last_error", "wm_workspace_bytes", "wm_create", "wm_destroy",
           "wm_apply_bc", "wm_compute_fluxes", "wm_compute_low_fluxes", "wm_limit_fluxes",
           "wm_rk3_update", "wm_enforce_admissible", "wm_update_prims", "wm_copy_old",
           "wm_get_dt", "wm_rhs_stage", "wm_step", "wm_init_dt", "wm_read_workspace", "wm_status",
           "wm_profile", "wm_profile_read", "wm_probe_fp64_flops", "wm_rhs_stage_static",
           "wm_solve_workspace_bytes", "wm_batch_create", "wm_batch_destroy", "wm_batch_set",
           "wm_batch_clear", "wm_batch_init_dt", "wm_batch_run", "wm_batch_query",
           "wm_batch_tile_shape", "wm_batch_scalars", "wm_batch_info", "wm_batch_profile",
           "wm_batch_profile_read", "wm_schlieren", "wm_copy_state", "wm_run", "wm_run_uses_graph",
           "wm_set_limiter_sweeps", "wm_batch_dt_log", "wm_verify_limiter_precheck",
           "wm_check_conversions", "wm_set_prechecks", "wm_verify_switch_precheck",
           "wm_check_sweep_arith", "wm_batch_spin_limit", "wm_verify_ducros_precheck")
STATIC_MAX_CELLS = 32768
PROF_GROUPS = ("bc", "prep", "faces", "limiter", "final")
BATCH_PHASES = ("bc_x", "bc_y", "prep", "sensor", "faces", "theta0", "theta1", "theta2", "final",
                "step_end")

_lib = None


class WavempError(RuntimeError):
    pass


def load(build_if_missing: bool = True) -> ctypes.CDLL:
    """Load libwavemp.so; build it first if it is missing or older than its sources."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if build_if_missing:
        path = _build.build()
    if not os.path.exists(path):
        raise WavempError(f"libwavemp.so not found at {path}; run wavemp._build.build()")
    L = ctypes.CDLL(path)
    vp, i, d = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
    P, F = ctypes.POINTER(WmParams), ctypes.POINTER(WmFields)
    L.wm_version.restype = ctypes.c_char_p
    L.wm_last_error.restype = ctypes.c_char_p
    L.wm_workspace_bytes.argtypes = [P, i, i, i]
    L.wm_workspace_bytes.restype = ctypes.c_size_t
    L.wm_create.argtypes = [P, i, i, i, vp, ctypes.c_size_t, ctypes.POINTER(vp)]
    L.wm_destroy.argtypes = [vp]
    L.wm_destroy.restype = None
    for name in ("wm_apply_bc", "wm_compute_fluxes", "wm_compute_low_fluxes",
                 "wm_enforce_admissible", "wm_update_prims", "wm_init_dt"):
        getattr(L, name).argtypes = [vp, F, vp]
    L.wm_limit_fluxes.argtypes = [vp, F, d, vp]
    L.wm_rk3_update.argtypes = [vp, F, F, d, d, d, vp]
    L.wm_copy_old.argtypes = [vp, F, F, vp]
    L.wm_get_dt.argtypes = [vp, F, ctypes.POINTER(d), vp]
    L.wm_rhs_stage.argtypes = [vp, F, F, d, d, d, vp]
    L.wm_step.argtypes = [vp, F, F, d, ctypes.POINTER(d), vp]
    L.wm_read_workspace.argtypes = [vp, i, vp, vp]
    L.wm_status.argtypes = [vp, ctypes.POINTER(WmStats), i, vp]
    L.wm_probe_fp64_flops.argtypes = [ctypes.POINTER(d), vp]
    L.wm_profile.argtypes = [vp, i]
    L.wm_rhs_stage_static.argtypes = [P, i, i, i, F, F, d, d, d, vp]
    L.wm_profile_read.argtypes = [vp, ctypes.POINTER(d * 5), ctypes.POINTER(ctypes.c_longlong * 5), i]
    BP = ctypes.POINTER(WmBatchParams)
    L.wm_solve_workspace_bytes.argtypes = [BP, i, i]
    L.wm_solve_workspace_bytes.restype = ctypes.c_size_t
    L.wm_batch_create.argtypes = [BP, i, ctypes.POINTER(vp)]
    L.wm_batch_destroy.argtypes = [vp]
    L.wm_batch_destroy.restype = None
    L.wm_batch_set.argtypes = [vp, i, ctypes.POINTER(WmSolveDesc), vp, ctypes.c_size_t]
    L.wm_batch_clear.argtypes = [vp, i]
    L.wm_batch_init_dt.argtypes = [vp, i, vp]
    L.wm_batch_run.argtypes = [vp, i, vp]
    L.wm_batch_query.argtypes = [vp, ctypes.POINTER(WmSolveStatus), vp]
    L.wm_batch_tile_shape.argtypes = [vp, i, i]
    L.wm_batch_scalars.argtypes = [vp, vp, i, vp]
    L.wm_batch_spin_limit.argtypes = [vp, ctypes.c_longlong]
    L.wm_batch_info.argtypes = [vp, ctypes.POINTER(i), ctypes.POINTER(i), ctypes.POINTER(i)]
    L.wm_batch_profile.argtypes = [vp, i]
    L.wm_schlieren.argtypes = [F, i, i, i, vp, vp, d, d, vp, vp, vp, vp]
    L.wm_copy_state.argtypes = [vp, vp, ctypes.c_longlong, vp]
    L.wm_run.argtypes = [vp, F, F, ctypes.POINTER(WmSchedule), ctypes.c_longlong, vp]
    L.wm_run_uses_graph.argtypes = [vp]
    L.wm_set_limiter_sweeps.argtypes = [vp, i]
    L.wm_batch_dt_log.argtypes = [vp, i, vp, ctypes.c_longlong, i]
    L.wm_set_prechecks.argtypes = [vp, i]
    L.wm_check_conversions.argtypes = [vp, ctypes.c_longlong, ctypes.POINTER(ctypes.c_longlong),
                                       ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong), vp]
    L.wm_check_sweep_arith.argtypes = [vp, ctypes.c_longlong, ctypes.POINTER(ctypes.c_longlong), vp]
    L.wm_verify_limiter_precheck.argtypes = [vp, F, d, ctypes.POINTER(ctypes.c_longlong),
                                             ctypes.POINTER(ctypes.c_longlong), vp]
    L.wm_verify_switch_precheck.argtypes = [vp, F, ctypes.POINTER(ctypes.c_longlong),
                                            ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong), vp]
    L.wm_verify_ducros_precheck.argtypes = [vp, F, ctypes.POINTER(ctypes.c_longlong),
                                            ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong), vp]
    L.wm_batch_profile_read.argtypes = [vp, ctypes.POINTER(d * len(BATCH_PHASES)), i, vp]
    for name in EXPORTS:
        if name not in ("wm_version", "wm_last_error", "wm_workspace_bytes", "wm_destroy",
                        "wm_solve_workspace_bytes", "wm_batch_destroy"):
            getattr(L, name).restype = i
    _lib = L
    return L


def check(rc: int, what: str):
    if rc != WM_OK:
        msg = _lib.wm_last_error().decode() if _lib is not None else ""
        raise WavempError(f"{what} failed: {WM_ERR.get(rc, rc)} {msg}")
