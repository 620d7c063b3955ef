#!/usr/bin/env python
"""Benchmark of the GB300 soap-bubble time step.

Workload (config c1): one bubble on the 512 x 1024 lat-long MAC grid,
radius 1, dt = 0.002 s, seeded thickness 1 + 0.2 SH(8..32), surfactant
1 + 0.01 U(-1,1), stream-function wind of max speed 1, velocities from zero,
mixed-precision PCG to relative residual 1e-6.  A step is one full time
step (Solver::stepForward of the reference).  Frames last 10 steps (t is the
frame start time, as in the reference's frame loop).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0).  value = cell-steps/s over all ranks with the
state resident in HBM (device time from CUDA events around every step, L2
flushed between steps); e2e = the same metric through the C ABI with the
step's wind forcing uploaded from pinned host memory and the thickness field
read back every step.  With N > 1 every rank steps its own independent
replica (the single-bubble step does not shard).

--impl reference times the CPU restatement of the reference step (the FP64
oracle, all host threads) on the same workload: the reference itself needs
AmgX, Boost and OpenCV and cannot be built here.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "cell-steps/s on 1 GB300 (plain vs batched mixed-prec @1e-6); p50/p99 latency"
UNIT = "cell-steps/s"
NTHETA, DT, RECIPE, SEED = 512, 0.002, "c1", 20261203
STEPS_PER_FRAME = 10
L2_FLUSH_BYTES = 512 << 20

# Algorithmic bytes per cell and launch (every array a kernel must read or
# write counted once; halo re-reads excluded)
# (FP32 = 4 B, map entry = 16 B: a float4 displacement).
ALG_BYTES_PER_CELL = {
    "k_advect_maps": 104,  # u_th,u_ph,fwd,bwd,gamma,uair0,corr_u,vair0,corr_v -> fwd',bwd',gamma',uair,vair
    "k_velocity": 16,      # u_th,u_ph -> u_th',u_ph'
    "k_bimocq": 56,        # eta,bwd',bwdprev,init,delta,initLast,deltaLast -> eta'
    "k_assemble": 44,      # eta',gamma',u_th',u_ph',uair,vair -> dmass,cE,cS,r0,b
    "k_post": 64,          # gamma',x,dx,xff(8),eta',u_th',u_ph',uair,vair -> gamma,dgamma,eta,deta,u_th,u_ph
    "k_accum": 80,         # eta_delta,gamma_delta,fwd',bwd',deta,dgamma,eta,gamma,eta_init,gamma_init
                           # -> eta_delta,gamma_delta,err_eta,err_gamma
    "k_reinit": 0,        # not counted: it corrects only on re-initialising steps (half the c1 run)
}
# The implicit solve, per cell.  Fixed: set-up (r0, rhs, dmass, cE, cS, the
# previous increment dx -> x (float-float), r, q, z or z1 = 44), the final true-residual check (x, r0,
# dmass, cE, cS -> r = 28) and the result (x, gamma_adv -> dx, gamma = 20).
# Per CG iteration: q = A p (z, p, dmass, cE, cS -> p, q = 28) and the update
# with the line solve (p, r, q, x -> x, r, z or z1 = 36).  With the Neumann
# term, one more phase per iteration and one at the start (z1, cS, r -> z =
# 16).  Keyed by the preconditioner a solve used (1: line, 2: Neumann).
PCG_BYTES = {1: (92, 64), 2: (108, 80)}
ROOFLINE_NOTES = {
    "k_solve": "latency-bound, not HBM-bound: the solve's vectors and factors stay in L2 and in "
               "shared memory across its iterations (DRAM traffic per launch is their first touch "
               "and does not grow with the iteration count); two grid barriers per CG iteration with the "
               "line blocks alone, three with the Neumann term",
}


def load_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        d = json.load(open(path))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def load_traffic():
    path = os.path.join(ROOT, "profiles", "traffic_c1.json")
    if os.path.exists(path):
        return json.load(open(path))
    return {}


class ClockSampler:
    """nvidia-smi clock / throttle samples while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.lines = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
            time.sleep(0.3)
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        return world, rank, local, dist
    return 1, 0, 0, None


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(x: float, dist) -> float:
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def state_mb() -> float:
    from soapbubble_gb300.bubble import bytes_required, make_params
    return bytes_required(make_params(NTHETA, DT)) / 1e6


def workload_config(extra=None):
    c = {"workload": "c1: single bubble, lat-long MAC grid 512 x 1024, radius 1, dt 0.002 s, "
                     "thickness 1+0.2*SH(8..32), surfactant 1+0.01*U(-1,1), wind max speed 1, "
                     "mixed-precision PCG to relative residual 1e-6",
         "nTheta": NTHETA, "nPhi": 2 * NTHETA, "cells": NTHETA * 2 * NTHETA, "dt": DT,
         "steps_per_frame": STEPS_PER_FRAME,
         "solver": "mixed-precision PCG (float-float iterate and scalars, exact dot-product sums, "
                   "float-float true-residual refinement); preconditioner: exact phi-line blocks, "
                   "plus their two-term Neumann series when the previous solve needed many "
                   "iterations",
         "solver_tol": 1e-6, "seed": SEED,
         "l2": f"flushed between timed steps ({L2_FLUSH_BYTES >> 20} MiB write); "
               f"state {state_mb():.0f} MB per bubble"}
    if extra:
        c.update(extra)
    return c


def cpu_oracle_rate(target_s: float, nthreads: int, max_steps: int = 1000, warmup: int = 0):
    """FP64 oracle (CPU restatement of the reference step) on the same
    workload: cell-steps/s over a bounded number of steps, after `warmup`
    untimed steps."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as po
    from soapbubble_gb300 import synth
    po.build()
    f = synth.make_fields(RECIPE, NTHETA, SEED)
    p = po.default_params(NTHETA, dt_s=DT)
    p.solver_tol = 1e-6
    p.nthreads = nthreads
    ob = po.OracleBubble(p, f.eta, f.gamma, f.uth, f.uph, f.uair_init, f.vair_init)
    k0 = 0
    for k0 in range(warmup):
        ob.p.t = (k0 // STEPS_PER_FRAME) * STEPS_PER_FRAME * DT
        ob.step()
    k0 = warmup
    t0 = time.perf_counter()
    ob.p.t = (k0 // STEPS_PER_FRAME) * STEPS_PER_FRAME * DT
    ob.step()  # first timed step: estimates the cost
    first = time.perf_counter() - t0
    n = max(1, min(max_steps, int(target_s / max(first, 1e-3))))
    t0 = time.perf_counter()
    for k in range(n):
        ob.p.t = ((k0 + 1 + k) // STEPS_PER_FRAME) * STEPS_PER_FRAME * DT
        ob.step()
    el = time.perf_counter() - t0
    cells = NTHETA * 2 * NTHETA
    return cells * n / el, n, el


def cuda_library_mapped() -> list:
    """Files of this repository's CUDA library mapped into this process."""
    try:
        with open("/proc/self/maps") as fh:
            return sorted({ln.split()[-1] for ln in fh if "libsoapbubble_gb300" in ln})
    except OSError:
        return []


def run_reference(args):
    world, rank, _, dist = dist_setup()
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    rate, n, el = cpu_oracle_rate(target_s=min(120.0, 20.0 + 2.0 * args.steps), nthreads=threads,
                                  max_steps=max(1, args.steps), warmup=args.warmup)
    mapped = cuda_library_mapped()
    if mapped:
        raise RuntimeError(f"the reference arm must not load the CUDA library: {mapped}")
    line = {
        "metric": METRIC, "value": rate, "unit": UNIT, "n_gpus": args.gpus, "steps": n,
        "requested_steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / n,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": workload_config(), "impl": "reference",
        "cpu_baseline": {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{n} steps of the 512x1024 workload after {args.warmup} "
                                   f"warm-up steps, FP64 oracle, OpenMP {threads} threads (the "
                                   "reference needs AmgX/Boost/OpenCV and cannot be built)"},
        "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_ours(args):
    world, rank, local, dist = dist_setup()
    from soapbubble_gb300 import build, cudart, synth
    from soapbubble_gb300.bubble import GpuBubble, make_params, stage_names
    build.build()
    cudart.set_device(local)
    names = stage_names()
    nst = len(names)
    f = synth.make_fields(RECIPE, NTHETA, SEED + rank)
    gb = GpuBubble(make_params(NTHETA, DT, solver_tol=1e-6, solver_mode=0, device=local))
    gb.upload_fields(f.eta, f.gamma, f.uth, f.uph, f.uair_init, f.vair_init)
    stream = gb.stream()
    flush = cudart.DeviceBuffer(L2_FLUSH_BYTES)
    N = NTHETA * 2 * NTHETA
    Nv = (NTHETA - 1) * 2 * NTHETA

    def t_of(k):
        return (k // STEPS_PER_FRAME) * STEPS_PER_FRAME * DT

    for k in range(args.warmup):
        gb.step(1, t_of(k), DT)
    gb.synchronize(require_converged=False)
    k0 = args.warmup
    launches0 = gb.stats().launches
    gb.reset_stats()  # failed solves and the worst residual of the timed steps
    ev = [(cudart.Event(), cudart.Event()) for _ in range(args.steps)]
    barrier(dist)
    gb.synchronize(require_converged=False)
    # timed region: K graph-launched steps, CUDA events on the bubble's
    # stream around every step, L2 flushed between steps (outside the events)
    with ClockSampler(local) as clocks:
        for k in range(args.steps):
            ev[k][0].record(stream)
            gb.step(1, t_of(k0 + k), DT)
            ev[k][1].record(stream)
            flush.memset_async(k & 0xff, stream)
        gb.synchronize(require_converged=False)
    barrier(dist)
    st = gb.stats()
    launches = st.launches - launches0
    total_ms = float(sum(a.elapsed_ms(b) for a, b in ev))
    total_ms_max = max_over_ranks(total_ms, dist)
    value = world * N * args.steps / (total_ms_max / 1e3)

    # per-kernel device times: a twin bubble replays the timed steps
    # (bit-identical trajectory) with CUDA events between its kernels; these
    # are the live input of the roofline
    kr = args.steps
    stage_ms = np.zeros(nst)
    iters, solve_bytes = [], []
    tw = GpuBubble(make_params(NTHETA, DT, solver_tol=1e-6, solver_mode=0, device=local))
    tw.upload_fields(f.eta, f.gamma, f.uth, f.uph, f.uair_init, f.vair_init)
    for k in range(args.warmup):
        tw.step(1, t_of(k), DT)
    tstream = tw.stream()
    for k in range(kr):
        tw.step_timed(1, t_of(k0 + k), DT, stage_ms)
        st_k = tw.stats()
        iters.append(st_k.solver_iters)
        fixed, per_it = PCG_BYTES[st_k.solver_precond_used]
        solve_bytes.append(fixed + per_it * st_k.solver_iters)
        flush.memset_async(k & 0xff, tstream)
    tw.synchronize(require_converged=False)
    tw.close()
    k_dom = int(np.argmax(stage_ms))
    dom = names[k_dom]
    mean_iters = float(np.mean(iters)) if iters else 0.0
    alg = dict(ALG_BYTES_PER_CELL)
    alg["k_solve"] = float(np.mean(solve_bytes)) if solve_bytes else 0.0
    per_launch_bytes = alg[dom] * N
    avg_launch_s = stage_ms[k_dom] / 1e3 / kr
    achieved = per_launch_bytes / avg_launch_s / 1e9
    peak, peak_kind = load_peaks()
    traffic = load_traffic().get(dom)
    # every stage against the same HBM peak (algorithmic bytes / live time)
    stage_roofline = {}
    for k_, n_ in enumerate(names):
        if stage_ms[k_] > 0 and alg.get(n_, 0) > 0:
            gbs = alg[n_] * N / (stage_ms[k_] / 1e3 / kr) / 1e9
            stage_roofline[n_] = {"achieved_gbs": round(gbs, 1), "frac": round(gbs / peak, 4)}
    stage_total = float(stage_ms.sum())
    stage_share = {n: round(float(m / stage_total), 4) for n, m in zip(names, stage_ms)}
    stage_us = {n: round(float(1e3 * m / kr), 2) for n, m in zip(names, stage_ms)}

    # end to end through the C ABI with pinned host buffers: a second twin
    # steps the same timed steps (same trajectory, same work per step), each
    # step uploading its wind forcing and copying the thickness back, which
    # the host reads.  The copies go through the C ABI's staged I/O (the
    # handle's copy stream), so step k+1's forcing and step k-1's thickness
    # move while step k computes; the host reads step k-1's thickness (two
    # host buffers) while step k runs.  The L2 flush between steps stays in
    # the compute stream and its device time (CUDA events) is taken out of
    # the host-clock total.
    e2e_steps = args.steps
    h_u = cudart.PinnedArray((N,))
    h_v = cudart.PinnedArray((Nv,))
    h_etas = [cudart.PinnedArray((N,)), cudart.PinnedArray((N,))]
    h_eta = h_etas[0]
    h_u.array[:] = f.uair_init.ravel().astype(np.float32)
    h_v.array[:] = f.vair_init.ravel().astype(np.float32)
    te = GpuBubble(make_params(NTHETA, DT, solver_tol=1e-6, solver_mode=0, device=local))
    te.upload_fields(f.eta, f.gamma, f.uth, f.uph, f.uair_init, f.vair_init)
    for k in range(args.warmup):
        te.step(1, t_of(k), DT)
    estream = te.stream()
    barrier(dist)
    te.synchronize(require_converged=False)
    fl_ev = [(cudart.Event(), cudart.Event()) for _ in range(e2e_steps)]
    readback = 0.0
    t0 = time.perf_counter()
    te.stage_upload_f32("uair_init", h_u.array)
    te.stage_upload_f32("vair_init", h_v.array)
    for k in range(e2e_steps):
        te.step(1, t_of(k0 + k), DT)  # takes the staged forcing of step k
        if k + 1 < e2e_steps:
            te.stage_upload_f32("uair_init", h_u.array)
            te.stage_upload_f32("vair_init", h_v.array)
        te.wait_staged()  # step k-1's thickness (and step k+1's forcing) landed
        if k > 0:  # the host reads step k-1's thickness while step k runs
            readback += float(h_etas[(k - 1) & 1].array[::4096].sum())
        te.stage_download_f32("eta", h_etas[k & 1].array)
        fl_ev[k][0].record(estream)
        flush.memset_async(k & 0xff, estream)
        fl_ev[k][1].record(estream)
    te.wait_staged()
    readback += float(h_etas[(e2e_steps - 1) & 1].array[::4096].sum())
    te.synchronize(require_converged=False)
    flush_s = sum(a.elapsed_ms(b) for a, b in fl_ev) / 1e3
    e2e_s = time.perf_counter() - t0 - flush_s
    h_eta = h_etas[(e2e_steps - 1) & 1]
    e2e_s_max = max_over_ranks(e2e_s, dist)
    e2e_value = world * N * e2e_steps / e2e_s_max
    finite = bool(np.isfinite(h_eta.array).all())
    final = gb.stats()
    same = bool(np.array_equal(te.download("eta"), gb.download("eta")))
    te.close()

    cpu = cpu1 = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        rate, n, el = cpu_oracle_rate(target_s=15.0, nthreads=threads)
        cpu = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{n} steps of the same 512x1024 workload (FP64 oracle, OpenMP "
                         f"{threads} threads, PCG to 1e-6), {el:.1f} s"}
        rate1, n1, el1 = cpu_oracle_rate(target_s=10.0, nthreads=1, max_steps=2)
        cpu1 = {"value": rate1, "unit": UNIT, "cores": 1, "kind": "port",
                "sample": f"{n1} steps of the same 512x1024 workload (FP64 oracle, one thread, "
                          f"PCG to 1e-6), {el1:.1f} s"}

    ensemble = serving = storage = whole = modes = None
    if rank == 0 and world == 1:
        h_u.free(); h_v.free(); [h.free() for h in h_etas]; flush.free()
        gb.close()
        gb = None
        from soapbubble_gb300 import c1report
        if args.whole_run_steps > 0:
            whole = c1report.whole_run(ALG_BYTES_PER_CELL, PCG_BYTES, peak, device=local,
                                       steps=args.whole_run_steps)
        if args.modes_prefix > 0:
            modes = c1report.solver_modes(prefix=args.modes_prefix, device=local,
                                          run_steps=max(args.whole_run_steps, args.modes_prefix))
        from soapbubble_gb300 import ensemble as ens, serve
        if args.ensemble_steps > 0:
            ensemble = ens.compare(steps=args.ensemble_steps, device=local)
        if args.serve_requests > 0:
            serving = serve.serve(args.serve_requests, 20.0, device=local)
            serving["sample"] = (f"first {args.serve_requests} requests of the seeded stream "
                                 "(python -m soapbubble_gb300.serve runs all 2000)")
        if args.storage_steps > 0:
            from soapbubble_gb300 import storage as stor
            storage = stor.compare(steps=args.storage_steps, device=local, peak_gbs=peak)

    ensemble_sharded = None
    if world > 1 and args.ensemble_steps > 0:
        # the ensemble's bubbles partitioned over the ranks (no data exchange)
        from soapbubble_gb300 import shard
        from soapbubble_gb300 import synth as syn
        r = shard.run_ensemble_shard(syn.ensemble(0), args.ensemble_steps, syn.ENSEMBLE["dt"],
                                     shard.Ranks(), device=local)
        ensemble_sharded = {
            "value": r["value"], "unit": UNIT, "ranks": world, "steps": args.ensemble_steps,
            "seconds_max": r["seconds_max"], "cells_x_steps": r["units"],
            "scaling": "strong (the 64-bubble ensemble split by cells over the ranks)",
            "path": "per rank: its members as one batched set, CUDA graph per step"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms_max / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": workload_config(),
            "parallelism": f"replicas x{world}" if world > 1 else "single",
            "state_mb": round(state_mb(), 1),
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak,
                         "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": traffic, "alg_bytes_per_launch": per_launch_bytes,
                         "avg_launch_us": avg_launch_s * 1e6,
                         "note": ROOFLINE_NOTES.get(dom, "")},
            "stage_roofline": stage_roofline,
            "cpu_baseline": cpu,
            "cpu_baseline_1thread": cpu1,
            "e2e": {"value": e2e_value, "unit": UNIT, "steps": e2e_steps,
                    "same_steps_as_value": same,
                    "h2d_bytes_per_step": 4 * (N + Nv), "d2h_bytes_per_step": 4 * N,
                    "inputs": "uair_init + vair_init (wind forcing) from pinned host memory",
                    "result": "eta (thickness) to pinned host memory, read by the host every step",
                    "overlap": "staged I/O on the handle's copy stream: step k+1's forcing and "
                               "step k-1's thickness move while step k computes; L2 flush "
                               "device time excluded"},
            "gpu_launches": int(launches),
            "clocks": clocks.summary(),
            "stage_share": stage_share, "stage_us_per_step": stage_us,
            "stage_steps": kr, "step_path": "CUDA graph per step (value); kernel-by-kernel with events (stages)",
            "solver_iters_mean": mean_iters, "solver_rel_resid_last": st.solver_rel_resid,
            "solver_nonconverged": int(st.solver_nonconverged),
            "solver_rel_resid_max": float(st.solver_rel_resid_max),
            "window": f"steps {k0}..{k0 + args.steps - 1} of the 1000-step run " + (
                "(the film is still whole; c1_whole_run covers the rupture)"
                if k0 + args.steps <= 330 else
                "(the film opens near step 330: the window includes the ruptured phase)"),
            "c1_whole_run": whole,
            "c1_solver_modes": modes,
            "solver_alg_bytes_per_cell": alg["k_solve"],
            "reinits": int(final.reinits), "result_finite": finite,
            "ensemble": ensemble,
            "serving": serving,
            "storage_c2": storage,
            "ensemble_sharded": ensemble_sharded,
        }
        print(json.dumps(line), flush=True)
    if gb is not None:
        h_u.free(); h_v.free(); [h.free() for h in h_etas]; flush.free()
        gb.close()
    if dist is not None:
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    # default: the whole c1 run (1000 steps; under gravity the film drains
    # and opens at the top after ~330 steps, and the solve then needs more
    # iterations)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    # the 64-bubble ensemble, plain vs batched (steps per member; 0 skips)
    ap.add_argument("--ensemble-steps", type=int, default=200)
    # a sample of the serving stream (requests; 0 skips)
    ap.add_argument("--serve-requests", type=int, default=100)
    # c2 (1024 x 2048) with FP32 and with BF16 field storage (steps; 0 skips)
    ap.add_argument("--storage-steps", type=int, default=100)
    # the whole c1 run, every step timed (steps; 0 skips)
    ap.add_argument("--whole-run-steps", type=int, default=1000)
    # plain FP32 vs mixed solve on c1: steps compared with the oracle (0 skips)
    ap.add_argument("--modes-prefix", type=int, default=10)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
