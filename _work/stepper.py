"""Step one bubble of a benchmark configuration and print its diagnostics.

    python -m soapbubble_gb300.stepper --config c2 --steps 4 [--nTheta 1024]

Used for profiling captures and quick checks of a configuration.
"""
from __future__ import annotations

import argparse
import json
import time

from . import build, synth
from .bubble import GpuBubble, make_params


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", default="c2", choices=sorted(synth.CONFIGS))
    ap.add_argument("--nTheta", type=int, default=0)
    ap.add_argument("--steps", type=int, default=4)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--solver-mode", type=int, default=0)
    ap.add_argument("--tol", type=float, default=1e-6)
    args = ap.parse_args()
    build.build()
    cfg = synth.CONFIGS[args.config]
    nT = args.nTheta or cfg["nTheta"]
    dt = cfg["dt"]
    f = synth.make_fields(cfg["recipe"], nT, args.seed)
    with GpuBubble(make_params(nT, dt, solver_tol=args.tol, solver_mode=args.solver_mode)) as gb:
        gb.upload_fields(f.eta, f.gamma, f.uth, f.uph, f.uair_init, f.vair_init)
        t0 = time.perf_counter()
        for k in range(args.steps):
            gb.step(1, (k // 10) * 10 * dt, dt)
        gb.synchronize()
        el = time.perf_counter() - t0
        s = gb.stats(mass=True)
        print(json.dumps({"config": args.config, "nTheta": nT, "steps": args.steps,
                          "ms_per_step": 1e3 * el / max(args.steps, 1),
                          "solver_iters": s.solver_iters, "rel_resid": s.solver_rel_resid,
                          "distortion": s.distortion, "reinits": s.reinits,
                          "mass_eta": s.mass_eta, "mass_gamma": s.mass_gamma}))
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
