"""Golden fixtures from the reference's own step code.

Runs the reference's kernel/*.cu (RiverIntheSky/SoapBubble), executed on the
host by oracle/ref/ (the CUDA launch syntax rewritten, the CUDA runtime,
AmgX, Boost and OpenCV replaced by shims; see oracle/ref/build_ref.py), on
seeded inputs, and stores the inputs with the reference's outputs:

  ref_c0_16x32_r1.npz      config c0's recipe, radius 1, dt 0.005 s: the
                           state after steps 1 and 4
  ref_cfg_32x64_r005.npz   the shipped config.txt coefficients (radius 0.05,
                           dt 0.005 s, nondimensional step 0.1): after step
                           1, after step 4 and after a fractional step of
                           dt / 3 at the frame time 0.02 s (the frame loop's
                           last step when DT is not a multiple of dt)
  ref_viscous_16x32_r005.npz  as the first with VISCOUS on, radius 0.05
  tex_256x512.npz          the reference's init/midFrequency.exr (channel B)
                           and init/velocityfield_512.exr (channels G, R)
                           read and resampled to the config.txt grid (512 x
                           256) by the library's EXR reader
                           (sb_exr_load_resized), as FP32

The reference checkout is read where it lies (default /root/reference,
$SBREF_SOURCE); the fixtures travel with the tests.  Run:

    python tests/golden/make_ref_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [ROOT, os.path.join(ROOT, "oracle", "ref")]

STATE = ["eta", "gamma", "u_theta", "u_phi", "eta_delta", "gamma_delta", "fwd_t", "fwd_p",
         "bwd_t", "bwd_p", "bwdprev_t", "bwdprev_p"]


def ref_bubble(nT, dt, radius, fields, viscous=False):
    import pyref
    rb = pyref.RefBubble(nT, dt, radius=radius, viscous=viscous)
    rb.init_from_images(None, None)
    for name, a in [("eta", fields.eta), ("eta_init", fields.eta), ("eta_init_last", fields.eta),
                    ("gamma", fields.gamma), ("gamma_init", fields.gamma),
                    ("gamma_init_last", fields.gamma), ("u_theta", fields.uth),
                    ("u_phi", fields.uph), ("uair_init", fields.uair_init),
                    ("vair_init", fields.vair_init)]:
        rb.set(name, a)
    return rb


def run_case(name, nT, dt, radius, recipe, seed, schedule, viscous=False):
    """schedule: list of (t, dt_step, tag or None)."""
    from soapbubble_gb300 import synth
    f = synth.make_fields(recipe, nT, seed)
    rb = ref_bubble(nT, dt, radius, f, viscous)
    out = {"nTheta": nT, "dt": dt, "radius": radius, "viscous": int(viscous),
           "in_eta": f.eta, "in_gamma": f.gamma, "in_u_theta": f.uth, "in_u_phi": f.uph,
           "in_uair_init": f.uair_init, "in_vair_init": f.vair_init,
           "sched_t": np.array([s[0] for s in schedule]),
           "sched_dt": np.array([s[1] for s in schedule])}
    coef = rb.coefficients()
    for k, v in coef.items():
        out["coef_" + k] = v
    tags = []
    for t, step_dt, tag in schedule:
        rb.step(t, step_dt)
        if tag:
            tags.append(tag)
            for s in STATE:
                out[f"{tag}_{s}"] = rb.get(s)
    out["tags"] = np.array(tags)
    np.savez_compressed(os.path.join(HERE, name), **out)
    rb.close()
    print("wrote", name)


def texture_fixture():
    import ctypes as C
    from soapbubble_gb300 import build, _lib
    build.build()
    L = _lib.lib()
    ref = os.environ.get("SBREF_SOURCE", "/root/reference")
    W, Hh = 512, 256
    chans = {}
    for key, fname, ch in [("B", "midFrequency.exr", "B"), ("G", "velocityfield_512.exr", "G"),
                           ("R", "velocityfield_512.exr", "R")]:
        out = np.zeros(W * Hh)
        rc = L.sb_exr_load_resized(os.path.join(ref, "init", fname).encode(), ch.encode(), W, Hh,
                                   out.ctypes.data_as(C.POINTER(C.c_double)))
        assert rc == 0, L.sb_last_error()
        chans[key] = out.reshape(Hh, W).astype(np.float32)
    np.savez_compressed(os.path.join(HERE, "tex_256x512.npz"), thickness_B=chans["B"],
                        airflow_G=chans["G"], airflow_R=chans["R"])
    print("wrote tex_256x512.npz")


def main():
    dt = 0.005
    run_case("ref_c0_16x32_r1.npz", 16, dt, 1.0, "c0", 7,
             [(0.0, dt, "s1"), (0.0, dt, None), (0.0, dt, None), (0.0, dt, "s4")])
    run_case("ref_cfg_32x64_r005.npz", 32, dt, 0.05, "c0", 11,
             [(0.0, dt, "s1"), (0.0, dt, None), (0.0, dt, None), (0.0, dt, "s4"),
              (0.02, dt / 3, "frac")])
    run_case("ref_viscous_16x32_r005.npz", 16, dt, 0.05, "c0", 5,
             [(0.0, dt, "s1"), (0.0, dt, None), (0.0, dt, "s3")], viscous=True)
    texture_fixture()


if __name__ == "__main__":
    main()
