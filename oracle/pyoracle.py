"""ctypes wrapper of the FP64 oracle (liboracle.so) -- TEST INFRASTRUCTURE ONLY.

Used by tests/, __graft_entry__.smoke() and bench.py's CPU legs as the
checker or as the timed CPU restatement of the reference step.  Parity is
unpinned against the reference binary (see oracle.h).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")


def build(quiet: bool = True) -> str:
    """Compile liboracle.so with the Makefile next to this file."""
    out = subprocess.run(["make", "-C", HERE], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    return LIB_PATH


class Params(C.Structure):
    _fields_ = [
        ("nTheta", C.c_int), ("nPhi", C.c_int), ("radius", C.c_double), ("dt", C.c_double),
        ("t", C.c_double), ("M", C.c_double), ("Cr", C.c_double), ("gs", C.c_double),
        ("gammaMax", C.c_double), ("evapRate", C.c_double), ("W1", C.c_double),
        ("W2", C.c_double), ("blend", C.c_double), ("U", C.c_double), ("strict", C.c_int),
        ("force_reinit", C.c_int), ("solver_tol", C.c_double), ("solver_max_iter", C.c_int),
        ("nthreads", C.c_int), ("plain_advection", C.c_int), ("single_step_velocity", C.c_int),
        ("viscous", C.c_int), ("re", C.c_double),
    ]


_STATE_FIELDS = ["eta", "gamma", "uth", "uph", "eta_init", "eta_delta", "eta_initLast",
                 "eta_deltaLast", "gam_init", "gam_delta", "gam_initLast", "gam_deltaLast",
                 "fwd_t", "fwd_p", "bwd_t", "bwd_p", "bwdprev_t", "bwdprev_p",
                 "uair_init", "vair_init"]


class State(C.Structure):
    _fields_ = [(n, C.POINTER(C.c_double)) for n in _STATE_FIELDS]


class Stats(C.Structure):
    _fields_ = [("distortion", C.c_double), ("reinit", C.c_int), ("solver_iters", C.c_int),
                ("solver_rel_resid", C.c_double), ("broken_cells", C.c_int),
                ("floor_oob", C.c_int)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        P, S, T = C.POINTER(Params), C.POINTER(State), C.POINTER(Stats)
        dp = C.POINTER(C.c_double)
        L.sb_oracle_default_params.argtypes = [P, C.c_int] + [C.c_double] * 6
        L.sb_oracle_step.argtypes = [P, S, T]
        L.sb_oracle_step.restype = C.c_int
        L.sb_oracle_update_maps.argtypes = [P, S]
        L.sb_oracle_advection.argtypes = [P, S]
        L.sb_oracle_bodyforce.argtypes = [P, S, T]
        L.sb_oracle_bodyforce.restype = C.c_int
        L.sb_oracle_distortion.argtypes = [P, S, T]
        L.sb_oracle_reinit.argtypes = [P, S]
        L.sb_oracle_assemble.argtypes = [P, S, dp, dp, dp, dp, dp]
        L.sb_oracle_solve.argtypes = [P, dp, dp, dp, dp]
        L.sb_oracle_solve.restype = C.c_int
        L.sb_oracle_sample.argtypes = [P, C.c_int, dp, C.c_int, dp, dp]
        L.sb_oracle_trace.argtypes = [P, dp, dp, C.c_double, C.c_int, dp, dp]
        L.sb_oracle_sample_mapping.argtypes = [P, dp, dp, C.c_int, dp, dp]
        L.sb_oracle_airflow.argtypes = [P, dp, dp, dp, dp]
        L.sb_oracle_identity_map.argtypes = [C.c_int, C.c_int, dp, dp]
        L.sb_oracle_viscous_forces.argtypes = [P, dp, dp, dp, dp, dp, dp]
        _lib = L
    return _lib


def _p(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(C.POINTER(C.c_double))


def default_params(nTheta: int, radius: float = 1.0, H: float = 1e-6, Gamma_m: float = 1e-6,
                   T: float = 298.15, dt_s: float = 0.005, blend: float = 0.5) -> Params:
    p = Params()
    lib().sb_oracle_default_params(C.byref(p), nTheta, radius, H, Gamma_m, T, dt_s, blend)
    return p


class OracleBubble:
    """FP64 state of one bubble in the reference's layout (absolute maps)."""

    def __init__(self, params: Params, eta, gamma, uth, uph, uair_init, vair_init):
        self.p = params
        nT, nP = params.nTheta, params.nPhi
        f = lambda a, shape: np.ascontiguousarray(np.asarray(a, dtype=np.float64).reshape(shape)).copy()
        self.a = {}
        self.a["eta"] = f(eta, (nT, nP))
        self.a["gamma"] = f(gamma, (nT, nP))
        self.a["uth"] = f(uth, (nT - 1, nP))
        self.a["uph"] = f(uph, (nT, nP))
        for q in ("eta", "gam"):
            src = self.a["eta" if q == "eta" else "gamma"]
            self.a[q + "_init"] = src.copy()
            self.a[q + "_initLast"] = src.copy()
            self.a[q + "_delta"] = np.zeros((nT, nP))
            self.a[q + "_deltaLast"] = np.zeros((nT, nP))
        for m in ("fwd", "bwd", "bwdprev"):
            t, ph = np.zeros((nT, nP)), np.zeros((nT, nP))
            lib().sb_oracle_identity_map(nT, nP, _p(t), _p(ph))
            self.a[m + "_t"], self.a[m + "_p"] = t, ph
        self.a["uair_init"] = f(uair_init, (nT, nP))
        self.a["vair_init"] = f(vair_init, (nT - 1, nP))
        self.stats = Stats()

    def _state(self) -> State:
        s = State()
        for n in _STATE_FIELDS:
            setattr(s, n, _p(self.a[n]))
        return s

    def copy(self) -> "OracleBubble":
        o = OracleBubble.__new__(OracleBubble)
        o.p = Params.from_buffer_copy(self.p)
        o.a = {k: v.copy() for k, v in self.a.items()}
        o.stats = Stats()
        return o

    def step(self) -> Stats:
        s = self._state()
        lib().sb_oracle_step(C.byref(self.p), C.byref(s), C.byref(self.stats))
        return self.stats

    def update_maps(self):
        s = self._state()
        lib().sb_oracle_update_maps(C.byref(self.p), C.byref(s))

    def advection(self):
        s = self._state()
        lib().sb_oracle_advection(C.byref(self.p), C.byref(s))

    def bodyforce(self) -> Stats:
        s = self._state()
        lib().sb_oracle_bodyforce(C.byref(self.p), C.byref(s), C.byref(self.stats))
        return self.stats

    def distortion(self) -> float:
        s = self._state()
        lib().sb_oracle_distortion(C.byref(self.p), C.byref(s), C.byref(self.stats))
        return self.stats.distortion

    def reinit(self):
        s = self._state()
        lib().sb_oracle_reinit(C.byref(self.p), C.byref(s))

    def assemble(self):
        nT, nP = self.p.nTheta, self.p.nPhi
        N = nT * nP
        gamma = self.a["gamma"].copy()
        val, rhs = np.zeros(5 * N), np.zeros(N)
        uair, vair = np.zeros(N + 1), np.zeros((nT - 1) * nP + 1)
        s = self._state()
        lib().sb_oracle_assemble(C.byref(self.p), C.byref(s), _p(gamma), _p(val), _p(rhs),
                                 _p(uair), _p(vair))
        return dict(gamma=gamma, val=val.reshape(N, 5), rhs=rhs, uair=uair, vair=vair)

    def solve(self, val, rhs, x0):
        x = np.ascontiguousarray(x0, dtype=np.float64).copy().ravel()
        rel = C.c_double(0)
        it = lib().sb_oracle_solve(C.byref(self.p), _p(np.ascontiguousarray(val).ravel()),
                                   _p(np.ascontiguousarray(rhs).ravel()), _p(x), C.byref(rel))
        return x, it, rel.value


def sample(params: Params, kind: int, field: np.ndarray, coords: np.ndarray) -> np.ndarray:
    coords = np.ascontiguousarray(coords, dtype=np.float64)
    out = np.zeros(coords.shape[0])
    lib().sb_oracle_sample(C.byref(params), kind, _p(np.ascontiguousarray(field, dtype=np.float64)),
                           coords.shape[0], _p(coords), _p(out))
    return out


def trace(params: Params, uth, uph, dt: float, coords: np.ndarray) -> np.ndarray:
    coords = np.ascontiguousarray(coords, dtype=np.float64)
    out = np.zeros_like(coords)
    lib().sb_oracle_trace(C.byref(params), _p(np.ascontiguousarray(uth, dtype=np.float64)),
                          _p(np.ascontiguousarray(uph, dtype=np.float64)), dt,
                          coords.shape[0], _p(coords), _p(out))
    return out


def sample_mapping(params: Params, map_t, map_p, coords: np.ndarray) -> np.ndarray:
    coords = np.ascontiguousarray(coords, dtype=np.float64)
    out = np.zeros_like(coords)
    lib().sb_oracle_sample_mapping(C.byref(params), _p(np.ascontiguousarray(map_t)),
                                   _p(np.ascontiguousarray(map_p)), coords.shape[0],
                                   _p(coords), _p(out))
    return out


def identity_map(nTheta: int):
    nPhi = 2 * nTheta
    t, ph = np.zeros((nTheta, nPhi)), np.zeros((nTheta, nPhi))
    lib().sb_oracle_identity_map(nTheta, nPhi, _p(t), _p(ph))
    return t, ph


def viscous_forces(params: Params, uth, uph, eta):
    """div u, fv (u_theta faces, gravity included) and fu (u_phi faces) of the
    VISCOUS variant."""
    nT, nP = params.nTheta, params.nPhi
    c = [np.ascontiguousarray(a, dtype=np.float64).ravel() for a in (uth, uph, eta)]
    div, fv, fu = np.zeros(nT * nP), np.zeros((nT - 1) * nP), np.zeros(nT * nP)
    lib().sb_oracle_viscous_forces(C.byref(params), _p(c[0]), _p(c[1]), _p(c[2]), _p(div),
                                   _p(fv), _p(fu))
    return div.reshape(nT, nP), fv.reshape(nT - 1, nP), fu.reshape(nT, nP)
