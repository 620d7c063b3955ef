"""ctypes binding of libsoapbubble_gb300.so (include/soapbubble.h).

The library is the product: there is no CPU fallback.  Importing this module
without a built library raises, naming the build command.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libsoapbubble_gb300.so")

SB_OK, SB_ERR_INVALID, SB_ERR_CUDA, SB_ERR_OOM, SB_ERR_NOT_CONVERGED, SB_ERR_BROKEN, SB_ERR_IO = range(7)
SB_STORE_FP32, SB_STORE_BF16 = 0, 1

FIELDS = ["eta", "gamma", "u_theta", "u_phi",
          "eta_init", "eta_delta", "eta_init_last", "eta_delta_last",
          "gamma_init", "gamma_delta", "gamma_init_last", "gamma_delta_last",
          "fwd_t", "fwd_p", "bwd_t", "bwd_p", "bwdprev_t", "bwdprev_p",
          "uair_init", "vair_init", "uair", "vair"]
FIELD_ID = {n: i for i, n in enumerate(FIELDS)}
# sb_system_array: the implicit system of the most recent step
SYSTEM = ["eta_adv", "gamma_adv", "dmass", "w_east", "w_south", "r0", "rhs", "dx"]
SYSTEM_ID = {n: i for i, n in enumerate(SYSTEM)}


class SbParams(C.Structure):
    _fields_ = [
        ("radius", C.c_double), ("H", C.c_double), ("U", C.c_double), ("c_m", C.c_double),
        ("Gamma_m", C.c_double), ("T", C.c_double), ("Ds", C.c_double), ("rm", C.c_double),
        ("nTheta", C.c_int), ("dt", C.c_double), ("DT", C.c_double), ("frames", C.c_int),
        ("blendCoeff", C.c_double), ("device", C.c_int),
        ("gs_scale", C.c_double), ("M_scale", C.c_double), ("solver_mode", C.c_int),
        ("solver_tol", C.c_double), ("solver_max_iter", C.c_int), ("force_reinit", C.c_int),
        ("nu_scale", C.c_double), ("storage", C.c_int), ("plain_advection", C.c_int),
        ("single_step_velocity", C.c_int), ("viscous", C.c_int),
        ("write_velocity_frames", C.c_int), ("write_concentration_frames", C.c_int),
        ("solver_precond", C.c_int), ("solver_cold_start", C.c_int),
    ]


class SbStats(C.Structure):
    _fields_ = [
        ("distortion", C.c_double), ("reinit", C.c_int), ("solver_iters", C.c_int),
        ("solver_rel_resid", C.c_double), ("solver_converged", C.c_int),
        ("broken_cells", C.c_int), ("steps", C.c_longlong), ("reinits", C.c_longlong),
        ("mass_eta", C.c_double), ("mass_gamma", C.c_double), ("launches", C.c_longlong),
        ("solver_precond_used", C.c_int), ("solves", C.c_longlong),
        ("solver_nonconverged", C.c_longlong), ("solver_rel_resid_max", C.c_double),
    ]


class SoapBubbleError(RuntimeError):
    def __init__(self, code: int, what: str, msg: str):
        super().__init__(f"{what} failed with status {code}: {msg}")
        self.code = code


_lib = None


def lib() -> C.CDLL:
    """Load the CUDA library (no fallback: a missing library is an error)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(
            f"{LIB_PATH} is missing; build it with `python -m soapbubble_gb300.build` "
            "or __graft_entry__.build()")
    L = C.CDLL(LIB_PATH)
    P, S = C.POINTER(SbParams), C.POINTER(SbStats)
    H = C.c_void_p
    dp = C.POINTER(C.c_double)
    L.sb_default_params.argtypes = [P]
    L.sb_default_params.restype = None
    L.sb_create.argtypes = [P, C.POINTER(H)]
    L.sb_destroy.argtypes = [H]
    L.sb_upload_fields.argtypes = [H, dp, dp, dp, dp, dp, dp]
    L.sb_upload_field.argtypes = [H, C.c_int, dp, C.c_size_t]
    L.sb_download_field.argtypes = [H, C.c_int, dp, C.c_size_t]
    L.sb_field_size.argtypes = [H, C.c_int]
    L.sb_download_system.argtypes = [H, C.c_int, dp, C.c_size_t]
    L.sb_field_size.restype = C.c_size_t
    L.sb_step.argtypes = [H, C.c_int, C.c_double, C.c_double]
    L.sb_step_timed.argtypes = [H, C.c_int, C.c_double, C.c_double, dp]
    L.sb_autotune.argtypes = [H, C.c_double, C.c_double, C.POINTER(C.c_int)]
    L.sb_stage_count.argtypes = []
    L.sb_stage_count.restype = C.c_int
    L.sb_stage_name.argtypes = [C.c_int]
    L.sb_stage_name.restype = C.c_char_p
    fp = C.POINTER(C.c_float)
    L.sb_upload_field_f32.argtypes = [H, C.c_int, fp, C.c_size_t]
    L.sb_download_field_f32.argtypes = [H, C.c_int, fp, C.c_size_t]
    L.sb_synchronize.argtypes = [H]
    L.sb_reset_stats.argtypes = [H]
    L.sb_selftest_grid_barrier.argtypes = [H, C.c_int, C.c_uint]
    L.sb_get_stats.argtypes = [H, S]
    L.sb_update_mass.argtypes = [H]
    L.sb_write_thickness_exr.argtypes = [H, C.c_char_p, C.POINTER(C.c_int)]
    L.sb_run.argtypes = [H, C.c_char_p, C.c_int]
    L.sb_write_exr_gray.argtypes = [C.c_char_p, C.c_int, C.c_int, C.POINTER(C.c_float)]
    L.sb_write_exr_gray.restype = C.c_int
    L.sb_mass_integrals_noalloc.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                            C.c_void_p]
    L.sb_mass_integrals_noalloc.restype = C.c_int
    L.sb_bytes_required.argtypes = [P]
    L.sb_bytes_required.restype = C.c_size_t
    L.sb_stream.argtypes = [H]
    L.sb_stream.restype = C.c_void_p
    L.sb_last_error.argtypes = []
    L.sb_last_error.restype = C.c_char_p
    ip = C.POINTER(C.c_int)
    L.sb_batch_create.argtypes = [C.POINTER(H), C.c_int, C.POINTER(H)]
    L.sb_batch_destroy.argtypes = [H]
    L.sb_batch_step.argtypes = [H, C.c_int, C.c_double, C.c_double]
    L.sb_batch_step_timed.argtypes = [H, C.c_int, C.c_double, C.c_double, dp]
    L.sb_batch_step_each.argtypes = [H, C.c_int, dp, C.c_double]
    L.sb_batch_autotune.argtypes = [H, C.c_double, C.c_double, ip]
    L.sb_batch_synchronize.argtypes = [H]
    L.sb_batch_retire.argtypes = [H, C.c_int]
    L.sb_batch_stream.argtypes = [H]
    L.sb_batch_stream.restype = C.c_void_p
    L.sb_init_thickness_from_exr.argtypes = [H, C.c_char_p]
    L.sb_init_airflow_from_exr.argtypes = [H, C.c_char_p]
    L.sb_exr_load_resized.argtypes = [C.c_char_p, C.c_char_p, C.c_int, C.c_int, dp]
    fp = C.POINTER(C.c_float)
    L.sb_stage_upload_f32.argtypes = [H, C.c_int, fp, C.c_size_t]
    L.sb_stage_download_f32.argtypes = [H, C.c_int, fp, C.c_size_t]
    L.sb_wait_staged.argtypes = [H]
    L.sb_write_velocity_exr.argtypes = [H, C.c_char_p]
    L.sb_write_concentration_exr.argtypes = [H, C.c_char_p]
    for name in ("sb_create", "sb_destroy", "sb_upload_fields", "sb_upload_field",
                 "sb_download_field", "sb_download_system", "sb_step", "sb_step_timed", "sb_autotune", "sb_upload_field_f32",
                 "sb_download_field_f32", "sb_synchronize", "sb_reset_stats",
                 "sb_selftest_grid_barrier", "sb_get_stats", "sb_update_mass", "sb_write_thickness_exr", "sb_run", "sb_batch_create",
                 "sb_batch_destroy", "sb_batch_step", "sb_batch_step_timed",
                 "sb_batch_step_each", "sb_batch_autotune", "sb_batch_synchronize", "sb_batch_retire",
                 "sb_init_thickness_from_exr", "sb_init_airflow_from_exr", "sb_exr_load_resized",
                 "sb_write_velocity_exr", "sb_write_concentration_exr", "sb_stage_upload_f32",
                 "sb_stage_download_f32", "sb_wait_staged"):
        getattr(L, name).restype = C.c_int
    _lib = L
    return L


def check(code: int, what: str) -> None:
    if code != SB_OK:
        raise SoapBubbleError(code, what, lib().sb_last_error().decode())


# Every symbol include/soapbubble.h declares (checked by the CPU tests).
EXPORTS = ["sb_default_params", "sb_create", "sb_destroy", "sb_upload_fields",
           "sb_upload_field", "sb_download_field", "sb_field_size", "sb_download_system", "sb_step",
           "sb_step_timed", "sb_autotune", "sb_stage_count", "sb_stage_name", "sb_upload_field_f32",
           "sb_download_field_f32", "sb_synchronize", "sb_reset_stats", "sb_selftest_grid_barrier",
           "sb_get_stats", "sb_update_mass", "sb_write_thickness_exr",
           "sb_run", "sb_write_exr_gray", "sb_mass_integrals_noalloc", "sb_bytes_required",
           "sb_stream", "sb_last_error", "sb_batch_create", "sb_batch_destroy", "sb_batch_step",
           "sb_batch_step_timed", "sb_batch_step_each", "sb_batch_autotune", "sb_batch_synchronize",
           "sb_batch_retire", "sb_batch_stream", "sb_init_thickness_from_exr", "sb_init_airflow_from_exr",
           "sb_exr_load_resized", "sb_write_velocity_exr", "sb_write_concentration_exr",
           "sb_stage_upload_f32", "sb_stage_download_f32", "sb_wait_staged"]
