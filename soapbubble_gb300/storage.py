"""FP32 against BF16 storage of the thickness and surfactant fields on the
c2 workload (one bubble, 1024 x 2048, dt 0.001 s, thickness 1 + 0.2 x a
blurred seeded 16 x 8 checkerboard, surfactant 1 + 0.05 SH(<= 16)).

Both runs start from the same fields and take the same steps; each reports
its device time per step (graph-launched steps between CUDA events; the
state of ~480 MB is far above L2, so no flush is needed), its per-stage
times with the algorithmic bytes each stage moves in that storage, and the
BF16 run's difference from the FP32 run at the end.

    python -m soapbubble_gb300.storage [--steps 100]
"""
from __future__ import annotations

import argparse
import json

import numpy as np

from . import cudart, synth
from .bubble import GpuBubble, bytes_required, make_params, stage_names

# Algorithmic bytes per cell and launch (every array once; FP32 = 4 B, map
# entry = 16 B, a stored field 4 or 2 B).  s = bytes of a stored element.
def alg_bytes(s: int) -> dict:
    return {
        "k_advect_maps": 100 + s,     # gamma sampled in the stored type; maps 16 B
        "k_velocity": 16,
        "k_bimocq": 44 + 3 * s,       # bwd', bwdprev (16 B), 2 deltas, eta_adv + eta, init, initL
        "k_assemble": 44,
        "k_post": 56 + 2 * s,         # eta, gamma written in the stored type; xff read
        "k_accum": 64 + 4 * s,        # deltas, maps (16 B), changes, errors + eta, gamma, inits
    }


def _rel(a: np.ndarray, b: np.ndarray) -> float:
    d = np.nanmax(np.abs(a - b))
    m = np.nanmax(np.abs(b))
    return float(d / m) if m > 0 else float(d)


def run(storage: int, steps: int, nTheta: int, seed: int, device: int = 0) -> dict:
    cfg = synth.CONFIGS["c2"]
    dt = cfg["dt"]
    f = synth.make_fields(cfg["recipe"], nTheta, seed)
    names = stage_names()
    N = nTheta * 2 * nTheta
    with GpuBubble(make_params(nTheta, dt, storage=storage, device=device)) as gb:
        gb.upload_fields(f.eta, f.gamma, f.uth, f.uph, f.uair_init, f.vair_init)
        t_of = lambda k: (k // 10) * 10 * dt
        for k in range(3):
            gb.step(1, t_of(k), dt)
        gb.synchronize(require_converged=False)
        s = gb.stream()
        a, b = cudart.Event(), cudart.Event()
        a.record(s)
        for k in range(steps):
            gb.step(1, t_of(3 + k), dt)
        b.record(s)
        gb.synchronize(require_converged=False)
        ms = a.elapsed_ms(b) / steps
        kr = min(steps, 20)
        st = np.zeros(16)
        for k in range(kr):
            gb.step_timed(1, t_of(3 + steps + k), dt, st)
        gb.synchronize(require_converged=False)
        alg = alg_bytes(2 if storage == 1 else 4)
        stages = {}
        for i, n in enumerate(names):
            us = 1e3 * st[i] / kr
            e = {"us": round(us, 2)}
            if n in alg and us > 0:
                e["alg_bytes_per_cell"] = alg[n]
                e["achieved_gbs"] = round(alg[n] * N / (us * 1e-6) / 1e9, 1)
            stages[n] = e
        fields = {n: gb.download(n) for n in ("eta", "gamma", "u_theta", "u_phi")}
        stt = gb.stats()
        return {"ms_per_step": ms, "cell_steps_per_s": N / (ms * 1e-3), "stages": stages,
                "state_mb": bytes_required(make_params(nTheta, dt, storage=storage)) / 1e6,
                "solver_converged": int(stt.solver_converged), "reinits": int(stt.reinits),
                "_fields": fields}


def compare(steps: int = 100, nTheta: int = 1024, seed: int = 20261203, device: int = 0,
            peak_gbs: float | None = None) -> dict:
    fp32 = run(0, steps, nTheta, seed, device)
    bf16 = run(1, steps, nTheta, seed, device)
    diff = {n: _rel(bf16["_fields"][n], fp32["_fields"][n]) for n in fp32["_fields"]}
    for r in (fp32, bf16):
        del r["_fields"]
        if peak_gbs:
            for e in r["stages"].values():
                if "achieved_gbs" in e:
                    e["frac_of_peak"] = round(e["achieved_gbs"] / peak_gbs, 4)
    return {
        "workload": (f"c2: one bubble {nTheta} x {2 * nTheta}, dt 0.001 s, thickness 1 + 0.2 "
                     "blurred 16x8 checkerboard, surfactant 1 + 0.05 SH(<=16), wind max speed 1; "
                     f"{steps} graph steps after 3 warm-up steps, stages over 20 more"),
        "fp32": fp32, "bf16": bf16,
        "bf16_speedup": fp32["ms_per_step"] / bf16["ms_per_step"],
        "bf16_vs_fp32_after_run": diff,
        "note": "BF16 holds eta, gamma and the BIMOCQ reference fields; the BIMOCQ change "
                "accumulators and all arithmetic stay FP32. Error against the FP64 oracle: "
                "tests/test_gpu_storage.py",
    }


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--nTheta", type=int, default=1024)
    args = ap.parse_args()
    from . import build
    build.build()
    print(json.dumps(compare(args.steps, args.nTheta)))
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
