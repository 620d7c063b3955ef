"""ctypes access to oracle/_ref/libsbref.so: the reference's own step code
(RiverIntheSky/SoapBubble kernel/*.cu) executed on the host by the shims of
oracle/ref/.  Test infrastructure: it pins the FP64 oracle against the
reference and generates golden fixtures; nothing in the product uses it.

    sim = RefBubble(nTheta=32, dt=0.005, radius=1.0)
    sim.init_from_images(thickness_bgr, airflow_bgr)   # the reference's initialisers
    sim.set("gamma", g)                                 # or any buffer directly
    sim.step(t, dt)                                     # Solver::stepForward
    eta = sim.get("eta")
"""
from __future__ import annotations

import ctypes as C
import os
import sys
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import build_ref  # noqa: E402

_libs = {}

# buffers of the reference's Solver by name (rows of nPhi, unpitched)
SCALARS = ["eta", "gamma", "u_theta", "u_phi", "eta_init", "eta_delta", "eta_init_last",
           "eta_delta_last", "gamma_init", "gamma_delta", "gamma_init_last", "gamma_delta_last"]
MAPS = ["fwd_t", "fwd_p", "bwd_t", "bwd_p", "bwdprev_t", "bwdprev_p"]
OTHER = ["uair_init", "vair_init", "uair", "vair", "rhs", "val"]


def available() -> bool:
    return build_ref.available() or os.path.exists(build_ref.LIB)


def lib(variant: str = "default") -> C.CDLL:
    """The reference built with its default switches, or with VISCOUS on
    (variant "viscous")."""
    if variant not in _libs:
        if build_ref.available():
            build_ref.build(variant=variant)
        L = C.CDLL(build_ref.lib_path(variant))
        d, dp, fp, vp = C.c_double, C.POINTER(C.c_double), C.POINTER(C.c_float), C.c_void_p
        L.sbref_create.argtypes = [d, d, d, d, d, d, d, d, C.c_int, d, d, C.c_int, d]
        L.sbref_create.restype = vp
        L.sbref_destroy.argtypes = [vp]
        L.sbref_init_from_images.argtypes = [vp, fp, fp]
        L.sbref_step.argtypes = [vp, d, d]
        L.sbref_step.restype = C.c_int
        L.sbref_get.argtypes = [vp, C.c_char_p, dp]
        L.sbref_get.restype = C.c_longlong
        L.sbref_set.argtypes = [vp, C.c_char_p, dp]
        L.sbref_set.restype = C.c_longlong
        L.sbref_coefficients.argtypes = [vp, dp]
        L.sbref_broken.argtypes = [vp]
        L.sbref_broken.restype = C.c_int
        L.sbref_amgx_last_rel_resid.restype = d
        L.sbref_amgx_last_iters.restype = C.c_int
        _libs[variant] = L
    return _libs[variant]


class RefBubble:
    """The reference's Bubble + Solver (kernel/bubble.cu:2568-2704) on the host."""

    def __init__(self, nTheta: int, dt: float, radius: float = 0.05, H: float = 1e-6,
                 U: float = 1.0, c_m: float = 0.5, Gamma_m: float = 1e-6, T: float = 298.15,
                 Ds: float = 0.0, rm: float = 5e-9, DT: Optional[float] = None, frames: int = 1,
                 blendCoeff: float = 0.5, viscous: bool = False):
        self.nTheta, self.nPhi, self.dt = nTheta, 2 * nTheta, dt
        self.radius = radius
        self.L = lib("viscous" if viscous else "default")
        self.h = self.L.sbref_create(radius, H, U, c_m, Gamma_m, T, Ds, rm, nTheta, dt,
                                    DT if DT is not None else 4 * dt, frames, blendCoeff)

    def close(self):
        if self.h:
            self.L.sbref_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        self.close()

    def init_from_images(self, thickness_bgr=None, airflow_bgr=None) -> None:
        """Solver::initThicknessfromPic / initAirflowfromPic on images of
        nTheta x nPhi x 3 floats (B, G, R); None takes the no-image path."""
        keep = []

        def ptr(a):
            if a is None:
                return None
            a = np.ascontiguousarray(a, dtype=np.float32)
            assert a.shape == (self.nTheta, self.nPhi, 3)
            keep.append(a)
            return a.ctypes.data_as(C.POINTER(C.c_float))

        self.L.sbref_init_from_images(self.h, ptr(thickness_bgr), ptr(airflow_bgr))

    def get(self, name: str) -> np.ndarray:
        n = self.L.sbref_get(self.h, name.encode(), None)
        if n == 0:
            raise KeyError(name)
        out = np.empty(n, dtype=np.float64)
        self.L.sbref_get(self.h, name.encode(), out.ctypes.data_as(C.POINTER(C.c_double)))
        if name == "val":
            return out.reshape(-1, 5)
        return out.reshape(-1, self.nPhi)

    def set(self, name: str, a: np.ndarray) -> None:
        a = np.ascontiguousarray(a, dtype=np.float64).ravel()
        n = self.L.sbref_get(self.h, name.encode(), None)
        if n != a.size:
            raise ValueError(f"{name}: {a.size} values for {n}")
        self.L.sbref_set(self.h, name.encode(), a.ctypes.data_as(C.POINTER(C.c_double)))

    def step(self, t: float, dt: Optional[float] = None) -> bool:
        """Solver::stepForward with currentTimeGlobal = t; returns True when
        the solver flagged the film as broken (a failed solve)."""
        return bool(self.L.sbref_step(self.h, t, self.dt if dt is None else dt))

    def coefficients(self) -> dict:
        out = np.zeros(7)
        self.L.sbref_coefficients(self.h, out.ctypes.data_as(C.POINTER(C.c_double)))
        return dict(zip(["dt", "M", "Cr", "gs", "gammaMax", "evap", "blend"], out))

    def last_solve(self):
        return self.L.sbref_amgx_last_iters(), self.L.sbref_amgx_last_rel_resid()
