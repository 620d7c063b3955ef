"""Seeded synthetic initial fields for the soap-bubble benchmark configurations.

The reference initialises thickness and air flow from EXR textures
(kernel/initializer.cu:50-135).  The benchmark configurations replace those
with seeded analytic fields of the same layout:

* thickness (eta) and surfactant (gamma) at cell centres,
  theta = (i + 0.5) h, phi = j h, h = pi / nTheta;
* the initial air flow ``uair_init`` at u_phi faces, theta = (i + 0.5) h,
  phi = (j - 0.5) h, and ``vair_init`` at u_theta faces, theta = (i + 1) h,
  phi = j h (include/header.cuh:24-35 MAC offsets);
* film velocities start at zero.

Every field is row-major [theta][phi] float64.  One master seed gives
per-bubble seeds through splitmix64, and each field draws from its own
numpy PCG64 stream, so a bubble's fields do not depend on how many other
bubbles were generated.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

MASK64 = (1 << 64) - 1


def splitmix64(x: int) -> int:
    """One splitmix64 output for state ``x`` (Steele, Lea, Flood 2014)."""
    z = (x + 0x9E3779B97F4A7C15) & MASK64
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK64
    return z ^ (z >> 31)


def sub_seed(seed: int, k: int) -> int:
    return splitmix64((seed * 0x100000001B3 + k) & MASK64)


def _legendre_normalized(lmax: int, x: np.ndarray) -> dict:
    """Fully normalised associated Legendre functions P[l, m](x), 0 <= m <= l.

    Standard three-term recursion in l for fixed m, seeded by the sectoral
    terms (stable for the degrees used here)."""
    s = np.sqrt(np.maximum(0.0, 1.0 - x * x))
    P = {}
    pmm = np.full_like(x, math.sqrt(1.0 / (4.0 * math.pi)))
    for m in range(0, lmax + 1):
        if m > 0:
            pmm = -math.sqrt((2.0 * m + 1.0) / (2.0 * m)) * s * pmm
        P[(m, m)] = pmm
        if m + 1 <= lmax:
            P[(m + 1, m)] = math.sqrt(2.0 * m + 3.0) * x * pmm
        for l in range(m + 2, lmax + 1):
            a = math.sqrt((4.0 * l * l - 1.0) / (l * l - m * m))
            b = math.sqrt(((l - 1.0) ** 2 - m * m) / (4.0 * (l - 1.0) ** 2 - 1.0))
            P[(l, m)] = a * (x * P[(l - 1, m)] - b * P[(l - 2, m)])
    return P


@dataclass
class SHSeries:
    """A real spherical-harmonic series with N(0,1) coefficients."""

    lmin: int
    lmax: int
    seed: int
    coef: dict = field(default_factory=dict)

    def __post_init__(self):
        rng = np.random.Generator(np.random.PCG64(self.seed))
        for l in range(self.lmin, self.lmax + 1):
            for m in range(-l, l + 1):
                self.coef[(l, m)] = float(rng.standard_normal())

    def _theta_parts(self, theta: np.ndarray):
        P = _legendre_normalized(self.lmax, np.cos(theta))
        A, B = {}, {}
        for (l, m), c in self.coef.items():
            am = abs(m)
            term = P[(l, am)] * (c if m == 0 else c * math.sqrt(2.0))
            if m >= 0:
                A[am] = A.get(am, 0.0) + term
            else:
                B[am] = B.get(am, 0.0) + term
        return A, B

    def evaluate(self, theta: np.ndarray, phi: np.ndarray, dphi: bool = False) -> np.ndarray:
        """Values (or d/dphi) on the tensor grid theta[:, None] x phi[None, :]:
        sum over m of a_m(theta) cos(m phi) + b_m(theta) sin(m phi), as one
        matrix product of the theta factors and the phi factors."""
        A, B = self._theta_parts(theta)
        ms = sorted(set(A) | set(B))
        zero = np.zeros_like(theta)
        T = np.empty((theta.size, 2 * len(ms)))
        F = np.empty((2 * len(ms), phi.size))
        for k, m in enumerate(ms):
            T[:, 2 * k] = A.get(m, zero)
            T[:, 2 * k + 1] = B.get(m, zero)
            c, s = np.cos(m * phi), np.sin(m * phi)
            if dphi:
                F[2 * k], F[2 * k + 1] = -m * s, m * c
            else:
                F[2 * k], F[2 * k + 1] = c, s
        return T @ F

    def dtheta(self, theta: np.ndarray, phi: np.ndarray, step: float = 1e-6) -> np.ndarray:
        return (self.evaluate(theta + step, phi) - self.evaluate(theta - step, phi)) / (2 * step)


def _normalise(f: np.ndarray, amplitude: float) -> np.ndarray:
    m = float(np.max(np.abs(f)))
    return f * (amplitude / m) if m > 0 else f


def grid_angles(nTheta: int):
    nPhi = 2 * nTheta
    h = math.pi / nTheta
    i = np.arange(nTheta, dtype=np.float64)
    j = np.arange(nPhi, dtype=np.float64)
    return {
        "h": h,
        "theta_c": (i + 0.5) * h,
        "phi_c": j * h,
        "theta_v": (i[:-1] + 1.0) * h,      # u_theta faces
        "phi_u": (j - 0.5) * h,             # u_phi faces
    }


def wind_from_stream(nTheta: int, seed: int, lmax: int = 8, max_speed: float = 1.0):
    """Tangential curl r x grad(psi) of a seeded stream function.

    u_phi = d(psi)/d(theta), u_theta = -(1/sin theta) d(psi)/d(phi); scaled so
    that the largest speed at cell centres is ``max_speed``.  Returns
    (uair_init at u_phi faces [nTheta, nPhi], vair_init at u_theta faces
    [nTheta-1, nPhi])."""
    g = grid_angles(nTheta)
    psi = SHSeries(1, lmax, seed)
    up_c = psi.dtheta(g["theta_c"], g["phi_c"])
    ut_c = -psi.evaluate(g["theta_c"], g["phi_c"], dphi=True) / np.sin(g["theta_c"])[:, None]
    scale = max_speed / float(np.max(np.sqrt(up_c ** 2 + ut_c ** 2)))
    uair = psi.dtheta(g["theta_c"], g["phi_u"]) * scale
    vair = -psi.evaluate(g["theta_v"], g["phi_c"], dphi=True) / np.sin(g["theta_v"])[:, None] * scale
    return uair, vair


def _gauss_blur_periodic(f: np.ndarray, sigma: float) -> np.ndarray:
    """Separable Gaussian blur: periodic in phi, mirrored at the poles."""
    r = int(math.ceil(4 * sigma))
    x = np.arange(-r, r + 1, dtype=np.float64)
    k = np.exp(-0.5 * (x / sigma) ** 2)
    k /= k.sum()
    out = np.zeros_like(f)
    for o, w in zip(x.astype(int), k):
        out += w * np.roll(f, o, axis=1)
    padded = np.concatenate([out[r - 1::-1], out, out[:-r - 1:-1]], axis=0)
    res = np.zeros_like(out)
    for o, w in zip(x.astype(int), k):
        res += w * padded[r + o:r + o + f.shape[0]]
    return res


def checkerboard(nTheta: int, seed: int, n_theta_sq: int = 16, n_phi_sq: int = 8,
                 sigma: float = 2.0) -> np.ndarray:
    """A 16 x 8 (theta x phi) checkerboard with a seeded phase, blurred."""
    rng = np.random.Generator(np.random.PCG64(seed))
    nPhi = 2 * nTheta
    shift = int(rng.integers(0, nPhi))
    sign = 1.0 if rng.random() < 0.5 else -1.0
    i = np.arange(nTheta)[:, None]
    j = (np.arange(nPhi)[None, :] + shift) % nPhi
    board = ((i * n_theta_sq // nTheta) + (j * n_phi_sq // nPhi)) % 2
    board = sign * (2.0 * board - 1.0)
    return _gauss_blur_periodic(board.astype(np.float64), sigma)


@dataclass
class BubbleFields:
    nTheta: int
    eta: np.ndarray
    gamma: np.ndarray
    uth: np.ndarray
    uph: np.ndarray
    uair_init: np.ndarray
    vair_init: np.ndarray


def make_fields(recipe: str, nTheta: int, seed: int) -> BubbleFields:
    """Initial fields of one bubble.

    recipe "c0": eta = 1 + 0.1 * SH(l <= 4); "c1": eta = 1 + 0.2 * SH(8 <= l <= 32);
    both with gamma = 1 + 0.01 * U(-1, 1).  "c2": eta = 1 + 0.2 * blurred
    checkerboard, gamma = 1 + 0.05 * SH(l <= 16).  Wind: stream function of
    degree <= 8, max speed 1.  Velocities start at zero."""
    nPhi = 2 * nTheta
    g = grid_angles(nTheta)
    s_eta, s_gam, s_wind = sub_seed(seed, 1), sub_seed(seed, 2), sub_seed(seed, 3)
    if recipe in ("c0", "c3"):
        eta = 1.0 + _normalise(SHSeries(0, 4, s_eta).evaluate(g["theta_c"], g["phi_c"]), 0.1)
    elif recipe == "c1":
        eta = 1.0 + _normalise(SHSeries(8, 32, s_eta).evaluate(g["theta_c"], g["phi_c"]), 0.2)
    elif recipe == "c2":
        eta = 1.0 + 0.2 * _normalise(checkerboard(nTheta, s_eta), 1.0)
    else:
        raise ValueError(f"unknown recipe {recipe!r}")
    if recipe == "c2":
        gamma = 1.0 + _normalise(SHSeries(0, 16, s_gam).evaluate(g["theta_c"], g["phi_c"]), 0.05)
    else:
        rng = np.random.Generator(np.random.PCG64(s_gam))
        gamma = 1.0 + 0.01 * rng.uniform(-1.0, 1.0, size=(nTheta, nPhi))
    uair, vair = wind_from_stream(nTheta, s_wind)
    return BubbleFields(nTheta, np.ascontiguousarray(eta), np.ascontiguousarray(gamma),
                        np.zeros((nTheta - 1, nPhi)), np.zeros((nTheta, nPhi)),
                        np.ascontiguousarray(uair), np.ascontiguousarray(vair))


# Benchmark configurations: grid, dimensional time step (s), steps, recipe.
CONFIGS = {
    "c0": dict(nTheta=64, dt=0.005, steps=100, recipe="c0"),
    "c1": dict(nTheta=512, dt=0.002, steps=1000, recipe="c1"),
    "c2": dict(nTheta=1024, dt=0.001, steps=500, recipe="c2"),
}

# Physical parameters shared by the configurations (config.txt keys, radius 1).
PHYSICS = dict(radius=1.0, H=1e-6, U=1.0, c_m=0.5, Gamma_m=1e-6, T=298.15, Ds=0.0,
               rm=5e-9, blendCoeff=0.5)

# The batched ensemble: 64 bubbles, nTheta uniform over ENSEMBLE_SIZES, the
# thickness recipe, time step and solver of c0, 200 steps.
ENSEMBLE = dict(members=64, steps=200, dt=0.005, recipe="c0", sizes=(64, 128, 256, 512),
                spread=0.5)


@dataclass
class Member:
    """One ensemble bubble: grid, field seed and the scale factors of its
    gravity (gs_scale), air viscosity (nu_scale, through the drag
    coefficient) and Marangoni coefficient (M_scale)."""
    nTheta: int
    seed: int
    gs_scale: float
    nu_scale: float
    M_scale: float


def ensemble(seed: int = 0, members: int = ENSEMBLE["members"], sizes=ENSEMBLE["sizes"],
             spread: float = ENSEMBLE["spread"]) -> list:
    """Seeded ensemble members: nTheta uniform over `sizes`, each physical
    scale uniform in [1 - spread, 1 + spread], a field seed per member."""
    rng = np.random.Generator(np.random.PCG64(sub_seed(seed, 0xE5)))
    out = []
    for k in range(members):
        nT = int(sizes[int(rng.integers(len(sizes)))])
        gs, nu, M = rng.uniform(1.0 - spread, 1.0 + spread, size=3)
        out.append(Member(nT, sub_seed(seed, k), float(gs), float(nu), float(M)))
    return out
