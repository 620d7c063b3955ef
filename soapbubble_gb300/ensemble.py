"""The batched ensemble workload: many bubbles of uneven grid size and
physical coefficients, stepped two ways.

* plain: one bubble at a time, kernel by kernel on its own stream (no graph),
  the plain FP32 implicit solve, synchronised after every step -- the way a
  user of the reference steps one Solver after another;
* batched: every member in one set, one launch per stage for all members,
  the step captured in a CUDA graph, tile sizes chosen by the autotuner, the
  mixed-precision solve.

Throughput is cell-steps/s = sum over members of nTheta * nPhi * steps / time.
"""
from __future__ import annotations

import time
from typing import List, Optional

import numpy as np

from . import cudart, synth
from .bubble import GpuBatch, GpuBubble, make_params


def member_fields(members, recipe: str = synth.ENSEMBLE["recipe"]):
    """Initial fields of every member (seeded per member)."""
    return [synth.make_fields(recipe, m.nTheta, m.seed) for m in members]


def make_bubbles(members, fields, dt: float, solver_mode: int, device: int = 0) -> List[GpuBubble]:
    out = []
    for m, f in zip(members, fields):
        g = GpuBubble(make_params(m.nTheta, dt, solver_mode=solver_mode, gs_scale=m.gs_scale,
                                  nu_scale=m.nu_scale, M_scale=m.M_scale, device=device))
        g.upload_fields(f.eta, f.gamma, f.uth, f.uph, f.uair_init, f.vair_init)
        out.append(g)
    return out


def cells(members) -> int:
    return int(sum(2 * m.nTheta * m.nTheta for m in members))


def frame_time(k: int, dt: float, steps_per_frame: int = 10) -> float:
    return (k // steps_per_frame) * steps_per_frame * dt


def run_plain(bubbles: List[GpuBubble], steps: int, dt: float, warmup: int = 1) -> dict:
    """Every member stepped alone, kernel by kernel, one after the other."""
    ms = np.zeros(16)
    for g in bubbles:
        g.step_timed(warmup, frame_time(0, dt), dt, ms)
    t0 = time.perf_counter()
    for k in range(steps):
        t = frame_time(warmup + k, dt)
        for g in bubbles:
            g.step_timed(1, t, dt, ms)  # per-kernel launches, synchronises
    el = time.perf_counter() - t0
    n = sum(g.nTheta * g.nPhi for g in bubbles)
    return {"value": n * steps / el, "ms_per_step": 1e3 * el / steps, "seconds": el}


def run_batched(bubbles: List[GpuBubble], steps: int, dt: float, warmup: int = 3,
                autotune: bool = True) -> dict:
    """All members as one set: autotuned tiles, one CUDA graph per step,
    device time between CUDA events on the batch's stream."""
    with GpuBatch(bubbles) as batch:
        tiles = batch.autotune(frame_time(0, dt), dt) if autotune else None
        k0 = 3 if autotune else 0
        for k in range(warmup):
            batch.step(1, frame_time(k0 + k, dt), dt)
        batch.synchronize()
        stream = batch.stream()
        a, b = cudart.Event(), cudart.Event()
        a.record(stream)
        for k in range(steps):
            batch.step(1, frame_time(k0 + warmup + k, dt), dt)
        b.record(stream)
        batch.synchronize()
        ms = a.elapsed_ms(b)
    n = sum(g.nTheta * g.nPhi for g in bubbles)
    return {"value": n * steps / (ms / 1e3), "ms_per_step": ms / steps, "tiles": tiles}


def compare(steps: int = synth.ENSEMBLE["steps"], seed: int = 0, device: int = 0,
            members: Optional[list] = None) -> dict:
    """Plain vs batched on the seeded ensemble (same initial fields)."""
    dt = synth.ENSEMBLE["dt"]
    members = members if members is not None else synth.ensemble(seed)
    fields = member_fields(members)
    plain = make_bubbles(members, fields, dt, solver_mode=1, device=device)
    try:
        rp = run_plain(plain, steps, dt)
    finally:
        for g in plain:
            g.close()
    mixed = make_bubbles(members, fields, dt, solver_mode=0, device=device)
    try:
        rb = run_batched(mixed, steps, dt)
        st = [g.stats() for g in mixed]
    finally:
        for g in mixed:
            g.close()
    sizes = {}
    for m in members:
        sizes[m.nTheta] = sizes.get(m.nTheta, 0) + 1
    return {
        "workload": (f"{len(members)} bubbles, nTheta x 2 nTheta with nTheta uniform over "
                     f"{sorted(sizes)} (counts {dict(sorted(sizes.items()))}), seeded gravity / "
                     f"air viscosity / Marangoni scales +-50%, c0 fields per member, dt {dt} s"),
        "members": len(members), "cells": cells(members), "steps": steps,
        "batched": {**rb, "solver": "mixed precision (float-float dots, refinement) to 1e-6",
                    "path": "one set, one launch per stage, CUDA graph per step, autotuned tiles",
                    "solver_iters_last_max": int(max(s.solver_iters for s in st)),
                    "converged_last": bool(all(s.solver_converged == 1 for s in st))},
        "plain": {**rp, "solver": "plain FP32 to 1e-6",
                  "path": "one bubble at a time, kernel by kernel (no graph), synchronised"},
        "speedup": rb["value"] / rp["value"],
    }
