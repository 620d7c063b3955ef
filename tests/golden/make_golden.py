"""Generates the golden fixtures of the step (run from the repository root:
`python tests/golden/make_golden.py`).

The reference cannot run here (it needs AmgX, Boost and OpenCV), so these
fixtures are outputs of the FP64 oracle (oracle/oracle.cpp), which restates
the reference's step.  They pin the oracle against later edits and give the
GPU tests a fixed input/output pair.  Inputs are rounded to what the GPU
stores (FP32 fields, FP32 map offsets from the cell centre) so that GPU and
oracle start from identical values.

The synthetic inputs depend on the host's libm and numpy in their last bits,
so a rerun elsewhere rewrites the existing fixtures with slightly different
values: commit only the fixtures that a change adds (the committed ones are
the pin).
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [ROOT, os.path.join(ROOT, "oracle")]

import pyoracle as po  # noqa: E402
from soapbubble_gb300 import synth  # noqa: E402

MAPS = ("fwd", "bwd", "bwdprev")


def round_state(ob):
    nT, nP = ob.p.nTheta, ob.p.nPhi
    for k, v in ob.a.items():
        if k.endswith("_t") or k.endswith("_p"):
            continue
        v[...] = v.astype(np.float32).astype(np.float64)
    ii = np.arange(nT)[:, None] + 0.5
    jj = np.arange(nP)[None, :] + 0.0
    for m in MAPS:
        t, p = ob.a[m + "_t"], ob.a[m + "_p"]
        t[...] = ii + (t - ii).astype(np.float32)
        d = np.mod(p - jj, nP)
        d = np.where(d >= nT, d - nP, d)
        p[...] = np.mod(jj + d.astype(np.float32).astype(np.float64) + nP, nP)


def case(name, nT, recipe, dt, pre, t, seed, strict=0, force=-1, radius=1.0, plain=0, single=0,
         viscous=0):
    f = synth.make_fields(recipe, nT, seed)
    p = po.default_params(nT, radius=radius, dt_s=dt)
    p.nthreads = 1
    p.plain_advection, p.single_step_velocity, p.viscous = plain, single, viscous
    ob = po.OracleBubble(p, f.eta, f.gamma, f.uth, f.uph, f.uair_init, f.vair_init)
    for k in range(pre):
        p.t = t
        ob.step()
    round_state(ob)
    p.t = t
    p.strict = strict
    p.force_reinit = force
    # inputs are FP32-exact by construction (map points: centre + FP32 offset)
    inp = {}
    for k, v in ob.a.items():
        if k.endswith("_t") or k.endswith("_p"):
            inp["in_" + k] = v.copy()
        else:
            inp["in_" + k] = v.astype(np.float32)
    st = ob.step()
    out = {"out_" + k: v.copy() for k, v in ob.a.items() if k not in ("uair_init", "vair_init")}
    # meta: nT, dt (s), t, strict, force_reinit, reinit, distortion, radius and
    # the switches plain_advection, single_step_velocity, viscous
    meta = np.array([nT, dt, t, strict, force, st.reinit, st.distortion, radius, plain, single,
                     viscous], dtype=np.float64)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), meta=meta, **inp, **out)
    print(name, "reinit", st.reinit, "distortion", st.distortion, "iters", st.solver_iters)


if __name__ == "__main__":
    po.build()
    case("c0_16x32_step", 16, "c0", 0.005, 4, 1.0, 2024)
    case("c0_16x32_reinit", 16, "c0", 0.005, 4, 1.0, 2025, force=1)
    case("c2_16x32_strict", 16, "c2", 0.001, 3, 0.5, 2026, strict=1)
    case("c1_32x64_step", 32, "c1", 0.002, 3, 2.0, 2027)
    case("c0_16x32_viscous", 16, "c0", 0.005, 4, 1.0, 2028, radius=0.05, viscous=1)
    case("c0_16x32_plain_single", 16, "c0", 0.005, 4, 1.0, 2029, plain=1, single=1)
