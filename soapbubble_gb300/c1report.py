"""Config c1's reports beside the bench line: the whole 1000-step run and the
plain-FP32 against the mixed-precision solve.

c1 is one bubble on the 512 x 1024 grid, radius 1, dt 0.002 s, 1000 steps.
Under gravity the film drains and opens at the top after ~330 steps; the
implicit solve then needs tens of PCG iterations per step and the maps are
re-initialised almost every step, so a window of a few early steps says
little about the run's cost:

* whole_run(): every one of the 1000 steps timed with CUDA events (graph
  per step), with the per-stage times of the same trajectory (a twin
  stepped kernel by kernel), PCG iterations, re-initialisations and failed
  solves, and the dominant stage's HBM roofline over the run;
* solver_modes(): the same prefix of the run with the plain FP32 solve and
  with the mixed-precision solve: each field's error against the FP64
  oracle after the prefix, the drift of the mass integrals (sum of eta
  sin(theta), of gamma sin(theta)) over the prefix and over the whole run,
  and the speed of each mode.
"""
from __future__ import annotations

import os
import sys
import time

import numpy as np

from . import cudart, synth
from .bubble import GpuBubble, make_params, stage_names

NTHETA, DT, RECIPE, SEED = 512, 0.002, "c1", 20261203
STEPS, STEPS_PER_FRAME = 1000, 10


def t_of(k: int) -> float:
    return (k // STEPS_PER_FRAME) * STEPS_PER_FRAME * DT


def _bubble(mode: int, device: int) -> GpuBubble:
    f = synth.make_fields(RECIPE, NTHETA, SEED)
    gb = GpuBubble(make_params(NTHETA, DT, solver_tol=1e-6, solver_mode=mode, device=device))
    gb.upload_fields(f.eta, f.gamma, f.uth, f.uph, f.uair_init, f.vair_init)
    return gb


def whole_run(alg_bytes: dict, pcg_bytes: dict, peak_gbs: float, device: int = 0,
              steps: int = STEPS) -> dict:
    """The c1 run from its initial state, every step timed (graph per
    step; events around each step on the bubble's stream)."""
    N = NTHETA * 2 * NTHETA
    gb = _bubble(0, device)
    stream = gb.stream()
    ev = [(cudart.Event(), cudart.Event()) for _ in range(steps)]
    gb.reset_stats()
    for k in range(steps):
        ev[k][0].record(stream)
        gb.step(1, t_of(k), DT)
        ev[k][1].record(stream)
    gb.synchronize(require_converged=False)
    st = gb.stats(mass=True)
    ms = np.array([a.elapsed_ms(b) for a, b in ev])
    total_ms = float(ms.sum())
    gb.close()
    # the same trajectory kernel by kernel: stage times, iterations, bytes
    names = stage_names()
    stage_ms = np.zeros(len(names))
    tw = _bubble(0, device)
    iters, solve_bytes, reinits = [], [], 0
    for k in range(steps):
        tw.step_timed(1, t_of(k), DT, stage_ms)
        s = tw.stats()
        iters.append(s.solver_iters)
        fixed, per_it = pcg_bytes[s.solver_precond_used]
        solve_bytes.append(fixed + per_it * s.solver_iters)
        reinits += s.reinit
    tw.close()
    alg = dict(alg_bytes)
    alg["k_solve"] = float(np.mean(solve_bytes))
    k_dom = int(np.argmax(stage_ms))
    dom = names[k_dom]
    stages = {}
    for n, m in zip(names, stage_ms):
        d = {"us_per_step": round(1e3 * m / steps, 2), "share": round(float(m / stage_ms.sum()), 4)}
        if alg.get(n, 0) > 0:
            gbs = alg[n] * N / (m / 1e3 / steps) / 1e9
            d.update(achieved_gbs=round(gbs, 1), frac=round(gbs / peak_gbs, 4))
        stages[n] = d
    half = steps // 2
    return {
        "steps": steps, "value": N * steps / (total_ms / 1e3), "unit": "cell-steps/s",
        "ms_per_step": total_ms / steps,
        "ms_per_step_first_300": float(ms[:300].mean()) if steps >= 300 else None,
        "ms_per_step_last_half": float(ms[half:].mean()),
        "solver_iters_mean": float(np.mean(iters)), "solver_iters_max": int(np.max(iters)),
        "solver_nonconverged": int(st.solver_nonconverged),
        "solver_rel_resid_max": float(st.solver_rel_resid_max),
        "reinits": int(reinits), "dominant_kernel": dom,
        "dominant_roofline": stages[dom], "stages": stages,
        "mass_eta_end": st.mass_eta, "mass_gamma_end": st.mass_gamma,
        "path": "graph per step, CUDA events around each step (no L2 flush: the run as a user "
                "runs it); stages from a twin stepped kernel by kernel on the same trajectory",
    }


def _mass(eta: np.ndarray, gamma: np.ndarray) -> tuple:
    s = np.sin((np.arange(eta.shape[0]) + 0.5) * np.pi / eta.shape[0])[:, None]
    return float((eta * s).sum()), float((gamma * s).sum())


def solver_modes(prefix: int = 10, device: int = 0, oracle_threads: int = 0,
                 run_steps: int = STEPS) -> dict:
    """Plain FP32 PCG (solver_mode 1) against mixed precision (mode 0) on
    c1: field errors against the FP64 oracle after `prefix` steps, mass
    drift over the prefix (and the oracle's), mass drift over `run_steps`
    steps, and the device time per step of each mode over the run."""
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, os.path.join(root, "oracle"))
    import pyoracle as po  # the FP64 checker
    po.build()
    f = synth.make_fields(RECIPE, NTHETA, SEED)
    p = po.default_params(NTHETA, dt_s=DT)
    p.solver_tol = 1e-10
    p.nthreads = oracle_threads or (os.cpu_count() or 1)
    ob = po.OracleBubble(p, f.eta, f.gamma, f.uth, f.uph, f.uair_init, f.vair_init)
    m0 = _mass(ob.a["eta"], ob.a["gamma"])
    t0 = time.perf_counter()
    for k in range(prefix):
        ob.p.t = t_of(k)
        ob.step()
    oracle_s = time.perf_counter() - t0
    mo = _mass(ob.a["eta"], ob.a["gamma"])
    out = {"prefix_steps": prefix, "run_steps": run_steps, "oracle_tol": 1e-10,
           "oracle_mass_drift_prefix": {"eta": mo[0] / m0[0] - 1, "gamma": mo[1] / m0[1] - 1},
           "oracle_seconds": oracle_s}
    names = {"eta": "eta", "gamma": "gamma", "u_theta": "uth", "u_phi": "uph"}
    for mode, label in ((1, "plain_fp32"), (0, "mixed")):
        gb = _bubble(mode, device)
        gb.synchronize()
        g0 = gb.stats(mass=True)
        for k in range(prefix):
            gb.step(1, t_of(k), DT)
        gp = gb.stats(mass=True)
        err = {}
        for g, o in names.items():
            a, b = gb.download(g), ob.a[o]
            err[g] = float(np.nanmax(np.abs(a - b)) / np.nanmax(np.abs(b)))
        # the rest of the run, timed on the device
        stream = gb.stream()
        e0, e1 = cudart.Event(), cudart.Event()
        gb.reset_stats()
        e0.record(stream)
        for k in range(prefix, run_steps):
            gb.step(1, t_of(k), DT)
        e1.record(stream)
        gb.synchronize(require_converged=False)
        ge = gb.stats(mass=True)
        ms = e0.elapsed_ms(e1) / max(1, run_steps - prefix)
        out[label] = {
            "field_error_vs_fp64_oracle": err,
            "mass_drift_prefix": {"eta": gp.mass_eta / g0.mass_eta - 1,
                                  "gamma": gp.mass_gamma / g0.mass_gamma - 1},
            "mass_drift_run": {"eta": ge.mass_eta / g0.mass_eta - 1,
                               "gamma": ge.mass_gamma / g0.mass_gamma - 1},
            "ms_per_step_rest_of_run": ms,
            "cell_steps_per_s_rest_of_run": NTHETA * 2 * NTHETA / (ms / 1e3),
            "solver_nonconverged_rest_of_run": int(ge.solver_nonconverged),
            "solver_rel_resid_max_rest_of_run": float(ge.solver_rel_resid_max),
        }
        gb.close()
    out["note"] = ("mass drift: relative change of sum(eta sin theta) and sum(gamma sin theta); "
                   "evaporation removes thickness by design, so eta's drift is physical and the "
                   "comparison is between the modes and against the oracle over the prefix")
    return out
