"""GPU parity at the reference's own configuration and against the
reference's own outputs.

* The reference-made fixtures (tests/golden/ref_*.npz: RiverIntheSky/
  SoapBubble's kernel/*.cu run on the host, tests/golden/make_ref_golden.py)
  are replayed on the GPU: config c0 at radius 1, the shipped config.txt
  coefficients (radius 0.05, dt 0.005 s: a nondimensional step of 0.1) with
  a fractional frame step, and the VISCOUS variant.
* config.txt itself: nTheta 256, radius 0.05, dt 0.005 s, DT 0.02 s, the
  thickness from init/midFrequency.exr and the wind from
  init/velocityfield_512.exr (the fixture holds them resampled to 512 x 256
  by the library's reader; here they go through the library's texture
  initialisers from an EXR file), checked against the FP64 oracle one step
  at a time from a fresh state and after 30 steps, through sb_run's frame
  loop over three frames, and with a fractional last step (DT = 1/24 s).
* Config c0's 100 steps, the GPU re-synchronised with the oracle before
  every step and compared after it.
Tolerance: 1e-5 normwise relative error per field (change accumulators
against their field), 1e-4 cells for the characteristic maps.
"""
import os

import numpy as np
import pytest

import _parity as P
from _exr import write_exr_bgr

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FIELDS = ["eta", "gamma", "u_theta", "u_phi"]
MAPS = [("fwd_t", "fwd_p"), ("bwd_t", "bwd_p"), ("bwdprev_t", "bwdprev_p")]
TOL, MAP_TOL = 1e-5, 1e-4


def _gpu(nT, dt, radius, **kw):
    from soapbubble_gb300.bubble import GpuBubble, make_params
    return GpuBubble(make_params(nT, dt, radius=radius, solver_tol=1e-10, solver_max_iter=4000,
                                 **kw))


def _tag_schedule(g):
    """(t, dt, tag) of the fixture's schedule (see test_ref_pin_cpu)."""
    import test_ref_pin_cpu as T
    return [(float(t), float(d), T._tag_at(g, k))
            for k, (t, d) in enumerate(zip(g["sched_t"], g["sched_dt"]))]


@pytest.mark.parametrize("case", ["ref_c0_16x32_r1.npz", "ref_cfg_32x64_r005.npz",
                                  "ref_viscous_16x32_r005.npz"])
def test_gpu_matches_reference_outputs(gpulib, case):
    g = np.load(os.path.join(GOLDEN, case))
    nT, dt, r = int(g["nTheta"]), float(g["dt"]), float(g["radius"])
    with _gpu(nT, dt, r, viscous=int(g["viscous"])) as gb:
        gb.upload_fields(g["in_eta"], g["in_gamma"], g["in_u_theta"], g["in_u_phi"],
                         g["in_uair_init"], g["in_vair_init"])
        for t, d, tag in _tag_schedule(g):
            gb.step(1, t, d)
            if not tag:
                continue
            for k in FIELDS:
                e = P.rel_err(gb.download(k), g[f"{tag}_{k}"])
                assert e <= TOL, (case, tag, k, e)
            for k in ("eta_delta", "gamma_delta"):
                field = g[f"{tag}_{k.split('_')[0]}"]
                e = float(np.nanmax(np.abs(gb.download(k) - g[f"{tag}_{k}"])) /
                          np.nanmax(np.abs(field)))
                assert e <= TOL, (case, tag, k, e)
            for t_, p_ in MAPS:
                e = P.map_err_cells(gb.download(t_), gb.download(p_), g[f"{tag}_{t_}"],
                                    g[f"{tag}_{p_}"], nT)
                assert e <= MAP_TOL, (case, tag, t_, e)


# --- config.txt: nTheta 256, radius 0.05, dt 0.005 s, the shipped textures ---

NT, DT_S, RADIUS = 256, 0.005, 0.05


@pytest.fixture(scope="module")
def texture_path(tmp_path_factory):
    tex = np.load(os.path.join(GOLDEN, "tex_256x512.npz"))
    path = str(tmp_path_factory.mktemp("tex") / "textures.exr")
    write_exr_bgr(path, tex["thickness_B"], tex["airflow_G"], tex["airflow_R"], "float")
    return path, tex


def _config_bubble(texture_path, **kw):
    path, _ = texture_path
    gb = _gpu(NT, DT_S, RADIUS, **kw)
    gb.init_thickness_from_exr(path)
    gb.init_airflow_from_exr(path)
    return gb


def _oracle_of(oracle, gb):
    """The oracle at the GPU bubble's (FP32) state, with config.txt's
    coefficients."""
    p = oracle.default_params(NT, radius=RADIUS, dt_s=DT_S)
    p.solver_tol = 1e-12
    ob = oracle.OracleBubble(p, gb.download("eta"), gb.download("gamma"), gb.download("u_theta"),
                             gb.download("u_phi"), gb.download("uair_init"),
                             gb.download("vair_init"))
    P.sync_state(gb, ob)
    return ob


def _check(gb, ob, what):
    err = P.compare(gb, ob, FIELDS)
    for k in FIELDS:
        assert err[k] <= TOL, (what, k, err)
    for m in ("fwd", "bwd", "bwdprev"):
        assert err[m] <= MAP_TOL, (what, m, err)
    return err


def test_texture_initialisers_match_reference_formulas(gpulib, texture_path):
    """sb_init_thickness_from_exr / sb_init_airflow_from_exr on the
    config.txt textures give the fields the reference's initialisers give
    (their formulas are pinned against the reference's own code by
    tests/test_ref_pin_cpu.py)."""
    _, tex = texture_path
    B = tex["thickness_B"].astype(np.float64)
    G = tex["airflow_G"].astype(np.float64)
    R = tex["airflow_R"].astype(np.float64)
    with _config_bubble(texture_path) as gb:
        np.testing.assert_allclose(gb.download("eta"), (B - 0.5) * 0.3 + 0.5, rtol=1e-7)
        np.testing.assert_allclose(gb.download("eta_init"), gb.download("eta"), rtol=0)
        np.testing.assert_allclose(gb.download("uair_init"),
                                   0.5 * (G + np.roll(G, 1, axis=1)) * RADIUS, rtol=1e-7,
                                   atol=1e-12)  # FP32 storage
        np.testing.assert_allclose(gb.download("vair_init"), -0.5 * (R[:-1] + R[1:]) * RADIUS,
                                   rtol=1e-7, atol=1e-12)
        assert np.all(gb.download("gamma") == 1.0)  # Solver::Solver's gamma = 1


def test_config_txt_one_step_fresh_and_after_30(gpulib, oracle, texture_path):
    with _config_bubble(texture_path) as gb:
        ob = _oracle_of(oracle, gb)
        ob.p.t = 0.0
        ob.step()
        gb.step(1, 0.0, DT_S)
        _check(gb, ob, "fresh")
        for k in range(1, 31):  # the oracle runs on; frames of 4 steps
            ob.p.t = (k // 4) * 0.02
            ob.step()
        P.sync_state(gb, ob)
        t = (31 // 4) * 0.02
        ob.p.t = t
        ob.step()
        gb.step(1, t, DT_S)
        _check(gb, ob, "after 30 steps")


def test_config_txt_frames_through_run(gpulib, oracle, texture_path):
    """sb_run over three frames of DT = 0.02 s (four steps each, t held at
    the frame start) against the oracle stepped with the same bookkeeping."""
    with _config_bubble(texture_path, DT=0.02, frames=4) as gb:
        ob = _oracle_of(oracle, gb)
        gb.run(None, frames=4)
        T = 0.0
        for i in range(1, 4):
            tf = T
            while T + DT_S <= i * 0.02:
                ob.p.t = tf
                ob.step()
                T += DT_S
            T = i * 0.02
        assert gb.stats().steps == 12
        _check(gb, ob, "three frames")


def test_config_txt_fractional_last_step(gpulib, oracle, texture_path):
    """DT = 1/24 s with dt = 0.005 s: a frame of eight steps and one of
    DT - 8 dt (kernel/bubble.cu:2669-2678), all at the frame's start time."""
    DTf = 1.0 / 24.0
    with _config_bubble(texture_path, DT=DTf, frames=2) as gb:
        ob = _oracle_of(oracle, gb)
        gb.run(None, frames=2)
        T, n = 0.0, 0
        while T + DT_S <= DTf:
            ob.p.t = 0.0
            ob.step()
            T += DT_S
            n += 1
        assert n == 8 and T + 1e-7 < DTf
        ob.p.dt = (DTf - T) / RADIUS  # the fractional step, nondimensional
        ob.p.t = 0.0
        ob.step()
        assert gb.stats().steps == 9
        _check(gb, ob, "fractional step")


def test_c0_every_step_of_100(gpulib, oracle):
    """Config c0 (64 x 128, radius 1, dt 0.005 s, 100 steps): before every
    step the GPU takes the oracle's state, after it both are compared."""
    from soapbubble_gb300 import synth
    nT, dt = 64, 0.005
    f = synth.make_fields("c0", nT, 20261203)
    p = oracle.default_params(nT, dt_s=dt)
    p.solver_tol = 1e-12
    ob = oracle.OracleBubble(p, f.eta, f.gamma, f.uth, f.uph, f.uair_init, f.vair_init)
    worst = {k: 0.0 for k in FIELDS + ["fwd", "bwd", "bwdprev"]}
    with _gpu(nT, dt, 1.0) as gb:
        for k in range(100):
            P.sync_state(gb, ob)
            t = (k // 10) * 10 * dt
            ob.p.t = t
            ob.step()
            gb.step(1, t, dt)
            err = P.compare(gb, ob, FIELDS)
            for key in worst:
                worst[key] = max(worst[key], err[key])
    for k in FIELDS:
        assert worst[k] <= TOL, worst
    for m in ("fwd", "bwd", "bwdprev"):
        assert worst[m] <= MAP_TOL, worst
