"""Python mirror of the reference's Bubble / Solver / Quantity surface.

`GpuBubble` owns one sb_bubble handle (C ABI, include/soapbubble.h) and moves
fields in the reference's host layout (row-major [theta][phi] float64,
u_theta with nTheta-1 rows; maps as absolute grid coordinates).  `Bubble`
keeps the reference constructor (include/bubble.cuh:78-84) and run()
(kernel/bubble.cu:2607-2704).
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional

import numpy as np

from . import _lib
from ._lib import SbParams, SbStats, check, lib


def _dp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def default_params() -> SbParams:
    p = SbParams()
    lib().sb_default_params(C.byref(p))
    return p


def make_params(nTheta: int, dt: float, radius: float = 1.0, H: float = 1e-6,
                Gamma_m: float = 1e-6, T: float = 298.15, blendCoeff: float = 0.5,
                DT: Optional[float] = None, frames: int = 1, solver_mode: int = 0,
                solver_tol: float = 1e-6, solver_max_iter: int = 1000, force_reinit: int = 0,
                gs_scale: float = 0.0, M_scale: float = 0.0, nu_scale: float = 0.0,
                device: int = 0, storage: int = 0, plain_advection: int = 0,
                single_step_velocity: int = 0, viscous: int = 0,
                write_velocity_frames: int = 0, write_concentration_frames: int = 0,
                solver_precond: int = 0, solver_cold_start: int = 0) -> SbParams:
    p = default_params()
    p.nTheta, p.dt, p.radius, p.H, p.Gamma_m, p.T = nTheta, dt, radius, H, Gamma_m, T
    p.blendCoeff = blendCoeff
    p.DT = DT if DT is not None else 10 * dt
    p.frames = frames
    p.solver_mode, p.solver_tol, p.solver_max_iter = solver_mode, solver_tol, solver_max_iter
    p.force_reinit, p.gs_scale, p.M_scale, p.device = force_reinit, gs_scale, M_scale, device
    p.nu_scale = nu_scale
    p.storage = storage  # 0: FP32, 1: BF16 thickness / surfactant fields
    p.plain_advection = plain_advection            # 1: BIMOCQ off
    p.single_step_velocity = single_step_velocity  # 1: RUNGE_KUTTA off
    p.viscous = viscous                            # 1: VISCOUS on
    p.write_velocity_frames = write_velocity_frames
    p.write_concentration_frames = write_concentration_frames
    p.solver_precond = solver_precond  # 0 auto, 1 phi-line blocks, 2 with the Neumann term
    p.solver_cold_start = solver_cold_start  # 1: every solve from a zero increment
    return p


class GpuBubble:
    """One bubble resident on the GPU (Solver + Quantity of the reference)."""

    def __init__(self, params: SbParams):
        self.params = params
        h = C.c_void_p()
        check(lib().sb_create(C.byref(params), C.byref(h)), "sb_create")
        self.h = h
        self.nTheta = params.nTheta
        self.nPhi = 2 * params.nTheta

    def close(self) -> None:
        if self.h:
            lib().sb_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- fields -------------------------------------------------------------
    def shape(self, name: str):
        n = lib().sb_field_size(self.h, _lib.FIELD_ID[name])
        if name in ("u_theta", "vair_init"):
            return (self.nTheta - 1, self.nPhi)
        if name in ("uair", "vair"):
            return (n,)
        return (self.nTheta, self.nPhi)

    def upload_fields(self, eta=None, gamma=None, u_theta=None, u_phi=None,
                      uair_init=None, vair_init=None) -> None:
        arrs = []

        def conv(a):
            if a is None:
                return None
            a = np.ascontiguousarray(a, dtype=np.float64)
            arrs.append(a)
            return _dp(a)

        args = [conv(a) for a in (eta, gamma, u_theta, u_phi, uair_init, vair_init)]
        check(lib().sb_upload_fields(self.h, *args), "sb_upload_fields")

    def upload(self, name: str, a: np.ndarray) -> None:
        a = np.ascontiguousarray(a, dtype=np.float64).ravel()
        check(lib().sb_upload_field(self.h, _lib.FIELD_ID[name], _dp(a), a.size), "sb_upload_field")

    def download(self, name: str) -> np.ndarray:
        n = lib().sb_field_size(self.h, _lib.FIELD_ID[name])
        out = np.empty(n, dtype=np.float64)
        check(lib().sb_download_field(self.h, _lib.FIELD_ID[name], _dp(out), n), "sb_download_field")
        return out.reshape(self.shape(name))

    def download_system(self, name: str) -> np.ndarray:
        """One array of the last step's implicit system (sb_download_system):
        eta_adv, gamma_adv, dmass, w_east, w_south, r0, rhs or dx."""
        out = np.empty(self.nTheta * self.nPhi, dtype=np.float64)
        check(lib().sb_download_system(self.h, _lib.SYSTEM_ID[name], _dp(out), out.size),
              "sb_download_system")
        return out.reshape(self.nTheta, self.nPhi)

    # -- stepping -----------------------------------------------------------
    def step(self, n: int = 1, t: float = 0.0, dt: Optional[float] = None) -> None:
        check(lib().sb_step(self.h, n, t, self.params.dt if dt is None else dt), "sb_step")

    def step_timed(self, n: int, t: float, dt: float, stage_ms: np.ndarray) -> None:
        """sb_step_timed: adds per-stage device milliseconds into stage_ms."""
        assert stage_ms.dtype == np.float64 and stage_ms.size >= lib().sb_stage_count()
        check(lib().sb_step_timed(self.h, n, t, dt, _dp(stage_ms)), "sb_step_timed")

    def autotune(self, t: float, dt: float) -> list:
        """sb_autotune: picks each stage's tile size (three tuning steps
        advance the bubble); returns the chosen cells per block by stage."""
        out = (C.c_int * lib().sb_stage_count())()
        check(lib().sb_autotune(self.h, t, dt, out), "sb_autotune")
        return list(out)

    def init_thickness_from_exr(self, path: str) -> None:
        """Solver::initThicknessfromPic: eta from channel B of an EXR texture
        (resampled, eta = (C - 0.5) 0.3 + 0.5); '' keeps eta = 0.5."""
        check(lib().sb_init_thickness_from_exr(self.h, path.encode()), "sb_init_thickness_from_exr")

    def init_airflow_from_exr(self, path: str) -> None:
        """Solver::initAirflowfromPic: the initial wind from channels G, R of
        an EXR texture; '' gives zero wind."""
        check(lib().sb_init_airflow_from_exr(self.h, path.encode()), "sb_init_airflow_from_exr")

    def upload_f32(self, name: str, a: np.ndarray) -> None:
        """Asynchronous FP32 upload from a host buffer the caller keeps alive."""
        assert a.dtype == np.float32 and a.flags.c_contiguous
        check(lib().sb_upload_field_f32(self.h, _lib.FIELD_ID[name],
                                        a.ctypes.data_as(C.POINTER(C.c_float)), a.size),
              "sb_upload_field_f32")

    def download_f32(self, name: str, out: np.ndarray) -> None:
        """Asynchronous FP32 download; synchronize() before reading `out`."""
        assert out.dtype == np.float32 and out.flags.c_contiguous
        check(lib().sb_download_field_f32(self.h, _lib.FIELD_ID[name],
                                          out.ctypes.data_as(C.POINTER(C.c_float)), out.size),
              "sb_download_field_f32")

    def stage_upload_f32(self, name: str, a: np.ndarray) -> None:
        """Host -> device copy on the copy stream, taken by the next step."""
        assert a.dtype == np.float32 and a.flags.c_contiguous
        check(lib().sb_stage_upload_f32(self.h, _lib.FIELD_ID[name],
                                        a.ctypes.data_as(C.POINTER(C.c_float)), a.size),
              "sb_stage_upload_f32")

    def stage_download_f32(self, name: str, out: np.ndarray) -> None:
        """The field after the queued steps to `out`, on the copy stream;
        wait_staged() before reading `out`."""
        assert out.dtype == np.float32 and out.flags.c_contiguous
        check(lib().sb_stage_download_f32(self.h, _lib.FIELD_ID[name],
                                          out.ctypes.data_as(C.POINTER(C.c_float)), out.size),
              "sb_stage_download_f32")

    def wait_staged(self) -> None:
        check(lib().sb_wait_staged(self.h), "sb_wait_staged")

    def synchronize(self, require_converged: bool = True) -> None:
        """Waits for the queued work; raises SoapBubbleError (code
        SB_ERR_NOT_CONVERGED) when the last solve missed its tolerance,
        unless require_converged is False (callers that count failed
        solves through stats() instead)."""
        rc = lib().sb_synchronize(self.h)
        if rc == _lib.SB_ERR_NOT_CONVERGED and not require_converged:
            return
        check(rc, "sb_synchronize")

    def reset_stats(self) -> None:
        """Restarts solver_nonconverged and solver_rel_resid_max."""
        check(lib().sb_reset_stats(self.h), "sb_reset_stats")

    def stats(self, mass: bool = False) -> SbStats:
        if mass:
            check(lib().sb_update_mass(self.h), "sb_update_mass")
        s = SbStats()
        check(lib().sb_get_stats(self.h, C.byref(s)), "sb_get_stats")
        return s

    def write_thickness_exr(self, path: str) -> bool:
        broken = C.c_int(0)
        check(lib().sb_write_thickness_exr(self.h, path.encode(), C.byref(broken)),
              "sb_write_thickness_exr")
        return bool(broken.value)

    def write_velocity_exr(self, path: str) -> None:
        check(lib().sb_write_velocity_exr(self.h, path.encode()), "sb_write_velocity_exr")

    def write_concentration_exr(self, path: str) -> None:
        check(lib().sb_write_concentration_exr(self.h, path.encode()),
              "sb_write_concentration_exr")

    def run(self, out_dir: Optional[str], frames: int = 0) -> None:
        check(lib().sb_run(self.h, out_dir.encode() if out_dir else None, frames), "sb_run")

    def stream(self) -> int:
        return lib().sb_stream(self.h)


# The limits sb_batch_create enforces: at most 1024 members, and the sum
# over members of nTheta (2 nTheta + 256) below 2^32.
BATCH_MAX_MEMBERS = 1024
BATCH_MAX_WEIGHT = 1 << 32


def batch_weight(nTheta: int) -> int:
    return nTheta * (2 * nTheta + 256)


class GpuBatch:
    """An ensemble of GpuBubbles stepped together (sb_batch_*): one kernel
    launch per stage for all members, one CUDA graph per step.  The members
    stay owned by the caller; step them only through the batch while it
    exists, and synchronize() before reading their fields."""

    def __init__(self, members):
        self.members = list(members)
        arr = (C.c_void_p * len(self.members))(*[m.h.value for m in self.members])
        h = C.c_void_p()
        check(lib().sb_batch_create(arr, len(self.members), C.byref(h)), "sb_batch_create")
        self.h = h

    def close(self) -> None:
        if self.h:
            lib().sb_batch_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def step(self, n: int, t, dt: float) -> None:
        """n steps at frame time t (one float for every member, or one per
        member)."""
        if np.ndim(t) == 0:
            check(lib().sb_batch_step(self.h, n, float(t), dt), "sb_batch_step")
        else:
            ts = np.ascontiguousarray(t, dtype=np.float64)
            assert ts.size == len(self.members)
            check(lib().sb_batch_step_each(self.h, n, _dp(ts), dt), "sb_batch_step_each")

    def step_timed(self, n: int, t: float, dt: float, stage_ms: np.ndarray) -> None:
        assert stage_ms.dtype == np.float64 and stage_ms.size >= lib().sb_stage_count()
        check(lib().sb_batch_step_timed(self.h, n, t, dt, _dp(stage_ms)), "sb_batch_step_timed")

    def autotune(self, t: float, dt: float) -> list:
        """Picks each stage's tile size (three tuning steps advance the
        members); returns the chosen cells per block by stage."""
        out = (C.c_int * lib().sb_stage_count())()
        check(lib().sb_batch_autotune(self.h, t, dt, out), "sb_batch_autotune")
        return list(out)

    def synchronize(self) -> None:
        check(lib().sb_batch_synchronize(self.h), "sb_batch_synchronize")

    def retire(self, k: int) -> None:
        """sb_batch_retire: member k leaves the batch's work (no rebuild)."""
        check(lib().sb_batch_retire(self.h, k), "sb_batch_retire")

    def stream(self) -> int:
        return lib().sb_batch_stream(self.h)


def stage_names() -> list:
    return [lib().sb_stage_name(i).decode() for i in range(lib().sb_stage_count())]


def exr_load_resized(path: str, channel: str, width: int, height: int) -> np.ndarray:
    """One channel of an uncompressed EXR, resampled to width x height with
    the bilinear weights the reference's textures go through (host only)."""
    out = np.zeros((height, width))
    check(lib().sb_exr_load_resized(path.encode(), channel.encode(), width, height, _dp(out)),
          "sb_exr_load_resized")
    return out


def bytes_required(params: SbParams) -> int:
    return lib().sb_bytes_required(C.byref(params))


class Bubble:
    """The reference's Bubble(...) + run() (include/bubble.cuh:78-88)."""

    def __init__(self, radius=0.05, H=0.0000005, U=1.0, c_m=0.5, Gamma_m=0.000001, T=298.15,
                 Ds=0.01, rm=0.000000005, nTheta=128, dt=0.005, DT=1.0 / 24.0, frames=1000,
                 outputDir="../output/test/", thicknessImage="", device=0, AMGconfig="",
                 blendCoeff=0.5):
        p = default_params()
        p.radius, p.H, p.U, p.c_m, p.Gamma_m, p.T, p.Ds, p.rm = radius, H, U, c_m, Gamma_m, T, Ds, rm
        p.nTheta, p.dt, p.DT, p.frames = int(nTheta), dt, DT, frames
        p.device, p.blendCoeff = device, blendCoeff
        self.outputDir = outputDir
        self.thicknessImage = thicknessImage
        self.AMGconfig = AMGconfig
        self.gpu = GpuBubble(p)
        if thicknessImage:
            raise NotImplementedError("thickness images are not supported yet")

    def run(self) -> None:
        if self.outputDir:
            os.makedirs(self.outputDir, exist_ok=True)
        self.gpu.run(self.outputDir or None)


def read_config(path: str) -> dict:
    """The 17 positional "key value" pairs of config.txt (kernel/main.cu:20-36)."""
    toks = open(path).read().split()
    vals = toks[1::2]
    if len(vals) < 17:
        raise ValueError(f"{path}: expected 17 key/value pairs, found {len(vals)}")
    names = ["radius", "H", "U", "c_m", "Gamma_m", "T", "Ds", "rm", "nTheta", "dt", "DT",
             "frames", "outputDir", "thicknessImage", "AMGconfig", "blendCoeff", "device"]
    conv = {"nTheta": int, "frames": int, "device": int, "outputDir": str,
            "thicknessImage": str, "AMGconfig": str}
    cfg = {n: conv.get(n, float)(v) for n, v in zip(names, vals)}
    if cfg["thicknessImage"] == "null":
        cfg["thicknessImage"] = ""
    return cfg
