"""GPU parity: one CUDA step against the FP64 oracle on identical inputs.

Tolerance: the thickness, surfactant and both velocity
components match the FP64 oracle to <= 1e-5 normwise relative error
(max |gpu - oracle| / max |oracle|) per step.  The BIMOCQ accumulators
(delta buffers) are small differences of O(1) fields and are checked at
1e-4; map points at 1e-4 grid cells.  The implicit solve runs to a relative
residual of 1e-10 here so that the comparison measures the step, not the
solver tolerance.
"""
import glob
import os

import numpy as np
import pytest

import _parity as P

pytestmark = pytest.mark.gpu

TOL_FIELD = 1e-5
TOL_DELTA = 1e-4
TOL_MAP_CELLS = 1e-4
PHYS = ("eta", "gamma", "u_theta", "u_phi")


def new_pair(oracle, nT, recipe, dt, pre, t, seed, force=0, solver_mode=0, tol=1e-10,
             gs_scale=1.0, nu_scale=1.0, M_scale=1.0, otol=None):
    from soapbubble_gb300 import synth
    from soapbubble_gb300.bubble import GpuBubble, make_params
    f = synth.make_fields(recipe, nT, seed)
    op = oracle.default_params(nT, dt_s=dt)
    op.t = t
    op.force_reinit = {0: -1, 1: 0, 2: 1}[force]
    # the scale options: gravity and Marangoni linearly, the drag coefficient
    # as the square root of the air viscosity
    op.gs *= gs_scale
    op.M *= M_scale
    op.Cr *= np.sqrt(nu_scale)
    if otol is not None:
        op.solver_tol = otol
    ob = oracle.OracleBubble(op, f.eta, f.gamma, f.uth, f.uph, f.uair_init, f.vair_init)
    for _ in range(pre):
        ob.step()
    gb = GpuBubble(make_params(nT, dt, solver_tol=tol, solver_max_iter=2000,
                               force_reinit=force, solver_mode=solver_mode, gs_scale=gs_scale,
                               nu_scale=nu_scale, M_scale=M_scale))
    P.sync_state(gb, ob)
    return gb, ob


def check_errors(err):
    for k in PHYS:
        assert err[k] <= TOL_FIELD, (k, err[k])
    for k in ("eta_delta", "gamma_delta", "eta_delta_last", "gamma_delta_last"):
        assert err[k] <= TOL_DELTA, (k, err[k])
    for k in ("eta_init", "gamma_init", "eta_init_last", "gamma_init_last"):
        assert err[k] <= TOL_FIELD, (k, err[k])
    for k in ("fwd", "bwd", "bwdprev"):
        assert err[k] <= TOL_MAP_CELLS, (k, err[k])


CASES = [
    # (nT, recipe, dt, steps before, t, seed, force)
    (64, "c0", 0.005, 0, 0.0, 1234, 0),
    (64, "c0", 0.005, 5, 1.0, 1234, 0),
    (64, "c0", 0.005, 30, 2.5, 1234, 0),
    (64, "c0", 0.005, 5, 1.0, 1234, 2),
    (128, "c1", 0.002, 5, 0.5, 77, 0),
    (128, "c2", 0.001, 5, 0.5, 78, 0),
]

# Under gravity the radius-1 film drains: by ~140 steps of c0 the top has
# no film left (eta = 0), velocities there are NaN (the reference writes NaN
# where both neighbouring thicknesses vanish, bubble.cu:1849-1853) and the
# implicit system carries identity rows.  One step from such a state.
BROKEN_CASES = [(64, "c0", 0.005, 160, 0.8, 1234), (64, "c0", 0.005, 260, 1.3, 1234)]


@pytest.mark.parametrize("case", BROKEN_CASES, ids=lambda c: f"{c[0]}-{c[1]}-pre{c[3]}")
def test_step_matches_oracle_on_broken_film(oracle, gpulib, case):
    nT, recipe, dt, pre, t, seed = case
    gb, ob = new_pair(oracle, nT, recipe, dt, pre, t, seed)
    with gb:
        assert np.isnan(ob.a["uth"]).any() and (ob.a["eta"] == 0).any()
        st = ob.step()
        gb.step(1, t, dt)
        gs = gb.stats()
        assert gs.broken_cells == st.broken_cells
        assert gs.solver_converged == 1
        for k in PHYS:
            g, o = gb.download(k), ob.a[P.FIELD_MAP[k]]
            np.testing.assert_array_equal(np.isnan(g), np.isnan(o), err_msg=k)
            np.testing.assert_array_equal(g == 0, o == 0, err_msg=k)
            assert P.rel_err(g, o) <= TOL_FIELD, (k, P.rel_err(g, o))


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"{c[0]}-{c[1]}-pre{c[3]}-force{c[6]}")
def test_step_matches_oracle(oracle, gpulib, case):
    nT, recipe, dt, pre, t, seed, force = case
    gb, ob = new_pair(oracle, nT, recipe, dt, pre, t, seed, force)
    with gb:
        st = ob.step()
        gb.step(1, t, dt)
        gs = gb.stats()
        assert gs.solver_converged == 1
        assert gs.solver_rel_resid < 1e-7
        assert gs.reinit == st.reinit
        assert gs.distortion == pytest.approx(st.distortion, rel=1e-3, abs=1e-6)
        check_errors(P.compare(gb, ob))


# The benchmark grids themselves: c1 (512 x 1024) and c2 (1024 x 2048), one
# step from a state the oracle stepped once (oracle solve to 1e-11).
FULL_CASES = [(512, "c1", 0.002, 1, 0.0, 20261203), (1024, "c2", 0.001, 1, 0.0, 20261204)]


@pytest.mark.parametrize("case", FULL_CASES, ids=lambda c: f"{c[0]}-{c[1]}")
def test_full_size_step_matches_oracle(oracle, gpulib, case):
    nT, recipe, dt, pre, t, seed = case
    gb, ob = new_pair(oracle, nT, recipe, dt, pre, t, seed, otol=1e-11)
    with gb:
        st = ob.step()
        gb.step(1, t, dt)
        gs = gb.stats()
        assert gs.solver_converged == 1
        assert gs.reinit == st.reinit
        assert gs.distortion == pytest.approx(st.distortion, rel=1e-3, abs=1e-6)
        err = P.compare(gb, ob)
        for k in PHYS + ("eta_init", "gamma_init", "eta_init_last", "gamma_init_last"):
            assert err[k] <= TOL_FIELD, (k, err[k])
        for k in ("fwd", "bwd", "bwdprev"):
            assert err[k] <= TOL_MAP_CELLS, (k, err[k])
        # the BIMOCQ change accumulators hold a step or two of small changes
        # here (c2: dt 0.001 s), so they are measured against the field they
        # correct rather than against their own size
        for k, field in (("eta_delta", "eta"), ("gamma_delta", "gamma"),
                         ("eta_delta_last", "eta"), ("gamma_delta_last", "gamma")):
            d = np.nanmax(np.abs(gb.download(k) - ob.a[P.FIELD_MAP[k]]))
            assert d / np.nanmax(np.abs(ob.a[P.FIELD_MAP[field]])) <= TOL_FIELD, (k, d)


@pytest.mark.parametrize("scales", [(1.5, 0.5, 1.3), (0.5, 1.5, 0.6)])
def test_scaled_coefficients_match_oracle(oracle, gpulib, scales):
    """Per-bubble gravity, air viscosity and Marangoni scales (the batched
    ensemble's per-member coefficients) reach the step as in the oracle."""
    gs, nu, M = scales
    gb, ob = new_pair(oracle, 64, "c0", 0.005, 5, 1.0, 555, gs_scale=gs, nu_scale=nu, M_scale=M)
    with gb:
        ob.step()
        gb.step(1, 1.0, 0.005)
        assert gb.stats().solver_converged == 1
        err = P.compare(gb, ob, PHYS)
        for k in PHYS:
            assert err[k] <= TOL_FIELD, (k, err[k])


def test_plain_fp32_solver_matches_oracle(oracle, gpulib):
    gb, ob = new_pair(oracle, 64, "c0", 0.005, 5, 1.0, 321, solver_mode=1, tol=1e-6)
    with gb:
        ob.step()
        gb.step(1, 1.0, 0.005)
        gs = gb.stats()
        assert gs.solver_converged == 1 and gs.solver_rel_resid <= 1e-6
        err = P.compare(gb, ob, PHYS)
        for k in PHYS:
            assert err[k] <= TOL_FIELD, (k, err[k])


def test_trajectory_20_steps(oracle, gpulib):
    """Independent 20-step runs from the same state stay within tolerance."""
    gb, ob = new_pair(oracle, 64, "c0", 0.005, 0, 0.0, 99)
    with gb:
        for k in range(20):
            t = (k // 10) * 0.05
            ob.p.t = t
            ob.step()
            gb.step(1, t, 0.005)
        err = P.compare(gb, ob, PHYS)
        for k in PHYS:
            assert err[k] <= TOL_FIELD, (k, err[k])


# the oracle-made step fixtures (the reference-made ref_* and the texture
# fixture have their own tests)
GOLDEN = sorted(p for p in glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz"))
                if not os.path.basename(p).startswith(("ref_", "tex_")))


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(g) for g in GOLDEN])
def test_step_matches_golden(gpulib, path):
    from soapbubble_gb300.bubble import GpuBubble, make_params
    z = np.load(path)
    nT, dt, t, strict, force = z["meta"][:5]
    meta = z["meta"]
    radius, plain, single, visc = ((float(meta[7]), int(meta[8]), int(meta[9]), int(meta[10]))
                                   if len(meta) >= 11 else (1.0, 0, 0, 0))
    nT = int(nT)
    gb = GpuBubble(make_params(nT, float(dt), radius=radius, solver_tol=1e-10, solver_max_iter=2000,
                               force_reinit={-1: 0, 0: 1, 1: 2}[int(force)], plain_advection=plain,
                               single_step_velocity=single, viscous=visc))
    with gb:
        for gname, oname in P.FIELD_MAP.items():
            gb.upload(gname, z["in_" + oname].astype(np.float64))
        gb.step(1, float(t), float(dt))
        assert gb.stats().reinit == int(z["meta"][5])
        for gname in PHYS:
            e = P.rel_err(gb.download(gname), z["out_" + P.FIELD_MAP[gname]])
            # the strict fixture carries the reference's float intrinsics
            assert e <= (TOL_FIELD if not strict else 2e-5), (gname, e)


def test_uniform_film_without_forcing_is_steady(gpulib):
    from soapbubble_gb300.bubble import GpuBubble, make_params
    nT, nP = 32, 64
    gb = GpuBubble(make_params(nT, 0.005, gs_scale=1e-30, solver_tol=1e-10))
    with gb:
        z = np.zeros((nT, nP))
        gb.upload_fields(np.full((nT, nP), 0.8), np.full((nT, nP), 1.3), np.zeros((nT - 1, nP)),
                         z, z, np.zeros((nT - 1, nP)))
        gb.step(3, 0.0, 0.005)
        evap = -3e-8 * 1.0 / 1e-6 * 0.005
        np.testing.assert_allclose(gb.download("eta"), 0.8 + 3 * evap, atol=2e-7)
        np.testing.assert_allclose(gb.download("gamma"), 1.3, atol=2e-7)
        assert np.max(np.abs(gb.download("u_theta"))) < 1e-6
        assert np.max(np.abs(gb.download("u_phi"))) < 1e-6


# The reference's compile-time switches as runtime options: BIMOCQ off
# (advectionAllCentered, no maps) and RUNGE_KUTTA off (one-step velocity
# trace), alone and together, against the oracle built with the same
# switches.
SWITCHES = [(1, 0), (0, 1), (1, 1)]


@pytest.mark.parametrize("sw", SWITCHES, ids=lambda s: f"plain{s[0]}-single{s[1]}")
def test_switch_variants_match_oracle(oracle, gpulib, sw):
    from soapbubble_gb300 import synth
    from soapbubble_gb300.bubble import GpuBubble, make_params
    plain, single = sw
    nT, dt, seed = 64, 0.005, 4321
    f = synth.make_fields("c0", nT, seed)
    op = oracle.default_params(nT, dt_s=dt)
    op.t = 0.5
    op.plain_advection, op.single_step_velocity = plain, single
    ob = oracle.OracleBubble(op, f.eta, f.gamma, f.uth, f.uph, f.uair_init, f.vair_init)
    for _ in range(5):
        ob.step()
    gb = GpuBubble(make_params(nT, dt, solver_tol=1e-10, solver_max_iter=2000,
                               plain_advection=plain, single_step_velocity=single))
    try:
        P.sync_state(gb, ob)
        for k in range(3):
            gb.step(1, 0.5, dt)
            ob.step()
            err = P.compare(gb, ob, list(PHYS))
            for name in PHYS:
                assert err[name] <= TOL_FIELD, (k, name, err[name])
        if plain:
            # no maps: they stay the identity, and nothing is re-initialised
            assert err["fwd"] <= TOL_MAP_CELLS and err["bwd"] <= TOL_MAP_CELLS
            assert gb.stats().reinits == 0
    finally:
        gb.close()


# The VISCOUS variant (viscous stress forces in the system and the velocity
# update) against the oracle built with the same switch, at the reference's
# config radius (0.05 m: re = 2.5e-3, most forces at their clamp) and at 1 m.
@pytest.mark.parametrize("radius", [0.05, 1.0], ids=["r0.05", "r1"])
def test_viscous_variant_matches_oracle(oracle, gpulib, radius):
    from soapbubble_gb300 import synth
    from soapbubble_gb300.bubble import GpuBubble, make_params
    nT, dt, seed = 64, 0.005, 4322
    f = synth.make_fields("c0", nT, seed)
    op = oracle.default_params(nT, radius=radius, dt_s=dt)
    op.t = 0.5
    op.viscous = 1
    ob = oracle.OracleBubble(op, f.eta, f.gamma, f.uth, f.uph, f.uair_init, f.vair_init)
    for _ in range(5):
        ob.step()
    gb = GpuBubble(make_params(nT, dt, radius=radius, solver_tol=1e-10, solver_max_iter=2000,
                               viscous=1))
    try:
        P.sync_state(gb, ob)
        for k in range(3):
            gb.step(1, 0.5, dt)
            ob.step()
            err = P.compare(gb, ob, list(PHYS))
            for name in PHYS:
                assert err[name] <= TOL_FIELD, (k, name, err[name])
    finally:
        gb.close()


# The preconditioner settings of the implicit solve (the phi-line blocks
# alone, with the Neumann term, chosen per solve) reach the same solution.
@pytest.mark.parametrize("precond", [0, 1, 2], ids=["auto", "line", "neumann"])
def test_preconditioner_settings_match_oracle(oracle, gpulib, precond):
    from soapbubble_gb300 import synth
    from soapbubble_gb300.bubble import GpuBubble, make_params
    nT, dt, seed = 64, 0.005, 4323
    f = synth.make_fields("c0", nT, seed)
    op = oracle.default_params(nT, dt_s=dt)
    op.t = 0.5
    ob = oracle.OracleBubble(op, f.eta, f.gamma, f.uth, f.uph, f.uair_init, f.vair_init)
    for _ in range(5):
        ob.step()
    gb = GpuBubble(make_params(nT, dt, solver_tol=1e-10, solver_max_iter=2000,
                               solver_precond=precond))
    try:
        P.sync_state(gb, ob)
        used = []
        for k in range(3):
            prev = gb.stats()
            gb.step(1, 0.5, dt)
            ob.step()
            st = gb.stats()
            assert st.solver_converged == 1
            used.append(st.solver_precond_used)
            if precond == 0 and k > 0:
                # the term comes on after a solve of 7 or more iterations
                # without it and goes off after one of 2 or fewer with it
                if prev.solver_precond_used == 1:
                    assert used[-1] == (2 if prev.solver_iters >= 7 else 1)
                else:
                    assert used[-1] == (1 if prev.solver_iters <= 2 else 2)
            err = P.compare(gb, ob, list(PHYS))
            for name in PHYS:
                assert err[name] <= TOL_FIELD, (k, name, err[name])
        if precond:
            assert used == [precond] * 3
        else:
            assert used[0] == 1  # a new bubble starts with the line blocks alone
    finally:
        gb.close()
