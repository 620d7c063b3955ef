"""Serving loop: bubble-simulation requests with continuous batching.

Requests arrive over time (seeded Poisson arrivals), each with its grid
size, step count, coefficients and initial fields (the payload).  The loop
admits waiting requests first come first served while their device memory
fits the HBM budget, keeps every admitted bubble resident, and steps all
resident bubbles together as one set (one launch per stage, one CUDA graph
per step; the set is rebuilt when requests join, and a finished request is
retired from it without a rebuild: the kernels skip it until the next
rebuild, when its bubble is freed).  Each member
runs at its own frame time.  Admission happens at frame boundaries (every
10 steps), so all members stay on the same frame grid; a thickness frame of
every member is streamed to the host every 10 of its steps, and its final
thickness when it completes.

A request's latency runs from its arrival to its final thickness on the
host.  Because a bubble stepped inside a set gives bit-identical results to
the same bubble stepped alone, the mix does not change any result.

Run a full stream from the command line, e.g.

    python -m soapbubble_gb300.serve --requests 2000 --rate 20
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import json
import os
import time
from dataclasses import dataclass
from typing import Dict, List, Optional

import numpy as np

from . import synth
from .bubble import (BATCH_MAX_MEMBERS, BATCH_MAX_WEIGHT, GpuBatch, GpuBubble, batch_weight,
                     bytes_required, make_params)

STEPS_PER_FRAME = 10
DT = synth.ENSEMBLE["dt"]


@dataclass
class Request:
    rid: int
    arrival: float        # seconds after the stream starts
    nTheta: int
    steps: int
    seed: int
    gs_scale: float
    nu_scale: float
    M_scale: float


def make_requests(n: int, rate: float, seed: int = 0, sizes=synth.ENSEMBLE["sizes"],
                  big: int = 1024, big_frac: float = 0.05, steps_range=(50, 500),
                  spread: float = synth.ENSEMBLE["spread"]) -> List[Request]:
    """n requests with exponential inter-arrival times (rate per second),
    nTheta uniform over `sizes` except a fraction `big_frac` at `big`, step
    counts uniform in steps_range, coefficient scales uniform in
    [1 - spread, 1 + spread], a field seed per request."""
    rng = np.random.Generator(np.random.PCG64(synth.sub_seed(seed, 0x5E)))
    t = 0.0
    out = []
    for k in range(n):
        t += float(rng.exponential(1.0 / rate))
        nT = big if rng.random() < big_frac else int(sizes[int(rng.integers(len(sizes)))])
        steps = int(rng.integers(steps_range[0], steps_range[1] + 1))
        gs, nu, M = rng.uniform(1.0 - spread, 1.0 + spread, size=3)
        out.append(Request(k, t, nT, steps, synth.sub_seed(seed, 1000 + k), float(gs), float(nu),
                           float(M)))
    return out


def payload(req: Request) -> synth.BubbleFields:
    return synth.make_fields(synth.ENSEMBLE["recipe"], req.nTheta, req.seed)


def params_of(req: Request, solver_mode: int = 0, device: int = 0):
    return make_params(req.nTheta, DT, solver_mode=solver_mode, gs_scale=req.gs_scale,
                       nu_scale=req.nu_scale, M_scale=req.M_scale, device=device)


def frame_time(k: int) -> float:
    return (k // STEPS_PER_FRAME) * STEPS_PER_FRAME * DT


@dataclass
class Active:
    req: Request
    bubble: GpuBubble
    done: int = 0                      # steps taken
    frame: Optional[np.ndarray] = None  # host buffer of the streamed frames


@dataclass
class Result:
    rid: int
    nTheta: int
    steps: int
    arrival: float
    admitted: float
    completed: float
    frames: int
    eta: Optional[np.ndarray] = None

    @property
    def latency(self) -> float:
        return self.completed - self.arrival


def run_alone(req: Request, fields, device: int = 0, keep_eta: bool = True) -> Result:
    """One request on its own: the same steps, frames and final download as
    in the serving loop (its isolated latency, measured from the call)."""
    t0 = time.perf_counter()
    g = GpuBubble(params_of(req, device=device))
    try:
        g.upload_fields(fields.eta, fields.gamma, fields.uth, fields.uph, fields.uair_init,
                        fields.vair_init)
        buf = np.empty(g.nTheta * g.nPhi, dtype=np.float32)
        k, frames = 0, 0
        while k < req.steps:
            n = min(STEPS_PER_FRAME - k % STEPS_PER_FRAME, req.steps - k)
            g.step(n, frame_time(k), DT)
            k += n
            if k % STEPS_PER_FRAME == 0 and k < req.steps:
                g.download_f32("eta", buf)
                g.synchronize(require_converged=False)
                frames += 1
        eta = g.download("eta")
    finally:
        g.close()
    t1 = time.perf_counter()
    return Result(req.rid, req.nTheta, req.steps, 0.0, 0.0, t1 - t0, frames,
                  eta if keep_eta else None)


class Server:
    """The serving loop over one GPU."""

    def __init__(self, budget_bytes: float = 150e9, device: int = 0, keep_eta: bool = False):
        self.budget = budget_bytes
        self.device = device
        self.keep_eta = keep_eta
        self.resident_bytes = 0
        self.max_resident = 0
        self.max_members = 0
        self.rebuilds = 0
        self.limit_waits = 0  # admissions deferred by the batch limits

    def run(self, requests: List[Request], payloads, clock_start: Optional[float] = None):
        """Serve `requests` (sorted by arrival).  `payloads` maps a request
        id to its fields.  Returns the results in request order."""
        pending = list(requests)
        waiting: List[Request] = []
        ready: List[Active] = []  # made while the GPU ran a frame, not yet in the set
        active: List[Active] = []
        members: List[Active] = []   # the batch's members in its order (retired ones too)
        retired: List[Active] = []   # finished, retired from the batch, freed at the next rebuild
        results: Dict[int, Result] = {}
        batch: Optional[GpuBatch] = None
        admitted_at: Dict[int, float] = {}
        changed = False
        g_step = 0
        cell_steps = 0
        t_start = time.perf_counter() if clock_start is None else clock_start

        def now():
            return time.perf_counter() - t_start

        def make_ready(in_use: bool) -> None:
            """Creates and fills the bubbles of waiting requests, first come
            first served, while they fit the budget (the first always does
            when nothing else is resident)."""
            while pending and pending[0].arrival <= now():
                waiting.append(pending.pop(0))
            while waiting:
                req = waiting[0]
                need = bytes_required(params_of(req, device=self.device))
                if self.resident_bytes + need > self.budget and (in_use or ready):
                    break
                # the batch's own limits (members, row tables): the request
                # waits until finished members have left the set
                if not fits_batch([a.req.nTheta for a in active + ready], req.nTheta):
                    self.limit_waits += 1
                    break
                waiting.pop(0)
                f = payloads[req.rid]
                g = GpuBubble(params_of(req, device=self.device))
                g.upload_fields(f.eta, f.gamma, f.uth, f.uph, f.uair_init, f.vair_init)
                ready.append(Active(req, g, 0, np.empty(g.nTheta * g.nPhi, dtype=np.float32)))
                self.resident_bytes += need

        try:
            while pending or waiting or ready or active:
                # admission at frame boundaries, first come first served: the
                # bubbles made during the last frame join, then any other
                # waiting request that fits
                if g_step % STEPS_PER_FRAME == 0:
                    make_ready(bool(active))
                    for a in ready:
                        admitted_at[a.req.rid] = now()
                        a.bubble.synchronize(require_converged=False)  # its fields are in place
                    if ready:
                        active.extend(ready)
                        ready.clear()
                        changed = True
                if not active:
                    g_step = 0  # idle: the frame grid restarts with the next admission
                    if pending and not waiting:
                        time.sleep(max(0.0, min(pending[0].arrival - now(), 0.05)))
                    continue
                if changed:
                    if batch is not None:
                        batch.close()
                    for a in retired:
                        a.bubble.close()
                        self.resident_bytes -= bytes_required(params_of(a.req, device=self.device))
                    retired.clear()
                    members = list(active)
                    batch = GpuBatch([a.bubble for a in members])
                    self.rebuilds += 1
                    changed = False
                    self.max_members = max(self.max_members, len(active))
                    self.max_resident = max(self.max_resident, self.resident_bytes)
                n = min(STEPS_PER_FRAME - g_step % STEPS_PER_FRAME,
                        min(a.req.steps - a.done for a in active))
                batch.step(n, [frame_time(a.done) for a in members], DT)
                g_step += n
                for a in active:
                    a.done += n
                    cell_steps += n * a.bubble.nTheta * a.bubble.nPhi
                if g_step % STEPS_PER_FRAME == 0:
                    # the next admission's bubbles are made while the GPU runs
                    make_ready(True)
                batch.synchronize()
                finished = []
                for a in active:
                    if a.done >= a.req.steps:
                        finished.append(a)
                    elif a.done % STEPS_PER_FRAME == 0:
                        a.bubble.download_f32("eta", a.frame)   # streamed frame
                for a in active:
                    if a.done < a.req.steps and a.done % STEPS_PER_FRAME == 0:
                        a.bubble.synchronize(require_converged=False)
                for a in finished:
                    eta = a.bubble.download("eta")
                    r = Result(a.req.rid, a.req.nTheta, a.req.steps, a.req.arrival,
                               admitted_at[a.req.rid], now(),
                               (a.req.steps - 1) // STEPS_PER_FRAME,
                               eta if self.keep_eta else None)
                    results[a.req.rid] = r
                if finished:
                    # retired from the batch in place; freed at the next rebuild
                    for a in finished:
                        batch.retire(next(k for k, m in enumerate(members) if m is a))
                        retired.append(a)
                    active = [a for a in active if a.done < a.req.steps]
                    if not active:
                        batch.close()
                        batch = None
                        for a in retired:
                            a.bubble.close()
                            self.resident_bytes -= bytes_required(params_of(a.req, device=self.device))
                        retired.clear()
                        members = []
        finally:
            if batch is not None:
                batch.close()
            for a in active + ready + retired:
                a.bubble.close()
        self.wall = now()
        self.cell_steps = cell_steps
        return [results[r.rid] for r in requests]


def fits_batch(member_nthetas: List[int], nTheta: int) -> bool:
    """Whether one more bubble of nTheta rows keeps a set of bubbles with
    member_nthetas within sb_batch_create's limits."""
    if len(member_nthetas) + 1 > BATCH_MAX_MEMBERS:
        return False
    w = sum(batch_weight(n) for n in member_nthetas) + batch_weight(nTheta)
    return w < BATCH_MAX_WEIGHT


def prepare_payloads(requests: List[Request], threads: int = 0) -> Dict[int, object]:
    """Every request's payload (its initial fields), computed by a thread
    pool before the stream starts: a request arrives with its payload, so
    preparing it is not part of the server's work."""
    threads = threads or min(16, os.cpu_count() or 1)
    with cf.ThreadPoolExecutor(max_workers=threads) as ex:
        fut = {r.rid: ex.submit(payload, r) for r in requests}
        return {k: f.result() for k, f in fut.items()}


def isolated_model(sizes, device: int = 0, steps: int = 60) -> Dict[int, dict]:
    """Measured single-request costs per grid size: set-up (create, upload,
    final download) and time per step including frame streaming, from one
    request of each size run alone; isolated latency = setup + steps * per_step."""
    out = {}
    for nT in sorted(set(sizes)):
        req = Request(-1, 0.0, nT, steps, 77 + nT, 1.0, 1.0, 1.0)
        f = payload(req)
        run_alone(req, f, device=device, keep_eta=False)           # warm (graph capture)
        short = Request(-1, 0.0, nT, STEPS_PER_FRAME, 77 + nT, 1.0, 1.0, 1.0)
        a = run_alone(short, f, device=device, keep_eta=False).completed
        b = run_alone(req, f, device=device, keep_eta=False).completed
        per_step = max(0.0, (b - a) / (steps - STEPS_PER_FRAME))
        out[nT] = {"setup_s": max(0.0, a - STEPS_PER_FRAME * per_step), "per_step_s": per_step}
    return out


def summarise(requests, results, server: Server, model=None) -> dict:
    lat = np.array([r.latency for r in results])
    out = {
        "requests": len(results),
        "rate_per_s": len(requests) / max(requests[-1].arrival, 1e-9),
        "wall_s": server.wall,
        "value": server.cell_steps / server.wall,
        "unit": "cell-steps/s",
        "latency_p50_s": float(np.percentile(lat, 50)),
        "latency_p99_s": float(np.percentile(lat, 99)),
        "latency_mean_s": float(lat.mean()),
        "max_resident_members": server.max_members,
        "admissions_deferred_by_batch_limits": server.limit_waits,
        "max_resident_gb": server.max_resident / 1e9,
        "budget_gb": server.budget / 1e9,
        "set_rebuilds": server.rebuilds,
    }
    if model:
        iso = np.array([model[r.nTheta]["setup_s"] + r.steps * model[r.nTheta]["per_step_s"]
                        for r in results])
        slow = lat / iso
        out.update({
            "isolated_p50_s": float(np.percentile(iso, 50)),
            "isolated_p99_s": float(np.percentile(iso, 99)),
            "p99_over_isolated_p99": float(np.percentile(lat, 99) / np.percentile(iso, 99)),
            "slowdown_p50": float(np.percentile(slow, 50)),
            "slowdown_p99": float(np.percentile(slow, 99)),
            "isolated_model": {str(k): v for k, v in model.items()},
        })
    return out


def serve(n: int, rate: float, seed: int = 0, budget_gb: float = 150.0, device: int = 0,
          model: bool = True) -> dict:
    reqs = make_requests(n, rate, seed)
    pay = prepare_payloads(reqs)
    srv = Server(budget_gb * 1e9, device=device)
    res = srv.run(reqs, pay)
    del pay
    mdl = isolated_model([r.nTheta for r in reqs], device=device) if model else None
    out = summarise(reqs, res, srv, mdl)
    out["workload"] = (f"{n} requests, Poisson arrivals at {rate}/s, nTheta uniform over "
                       f"{list(synth.ENSEMBLE['sizes'])} plus 5% at 1024, steps U[50, 500], "
                       f"c0 fields and +-50% coefficients per request, dt {DT} s, "
                       f"HBM budget {budget_gb} GB, a frame streamed every {STEPS_PER_FRAME} steps")
    return out


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--requests", type=int, default=2000)
    ap.add_argument("--rate", type=float, default=20.0)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--budget-gb", type=float, default=150.0)
    ap.add_argument("--device", type=int, default=0)
    args = ap.parse_args()
    from . import build
    build.build()
    print(json.dumps(serve(args.requests, args.rate, args.seed, args.budget_gb, args.device)))
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
