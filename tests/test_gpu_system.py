"""The implicit surfactant system as the GPU assembles it (sb_download_system)
against the reference's matrix (concentrationLinearSystemKernel,
kernel/bubble.cu:1301-1473, restated by the oracle), and the FP32 range
guard of its diagonal.

The library assembles the system for the increment dx = gamma_new -
gamma_adv (rows of cells with almost no surfactant scaled by powers of two;
none in the states compared coefficient by coefficient here).  The reference's row of an unbroken cell c is recovered from the
GPU arrays as: diagonal dmass_c + the stored weights to its unbroken
neighbours, off-diagonals -w (the stored weights; a weight towards a broken
neighbour sits in dmass instead), rhs b; r0 = b - A gamma_adv.  A broken
cell is the reference's identity row with rhs gmax.

Tolerance: FP32 assembly from FP32 inputs, 1e-5 relative per coefficient;
r0 (a difference of O(b) terms) 1e-5 of max |b|.
"""
import numpy as np
import pytest

import _parity as P

pytestmark = pytest.mark.gpu


def _pair(oracle, recipe, nT, dt, pre, t, seed, gamma_patch=None, force_reinit=0):
    from soapbubble_gb300 import synth
    from soapbubble_gb300.bubble import GpuBubble, make_params
    f = synth.make_fields(recipe, nT, seed)
    op = oracle.default_params(nT, dt_s=dt)
    op.t = t
    ob = oracle.OracleBubble(op, f.eta, f.gamma, f.uth, f.uph, f.uair_init, f.vair_init)
    for _ in range(pre):
        ob.step()
    if gamma_patch is not None:
        gamma_patch(ob)
    gb = GpuBubble(make_params(nT, dt, solver_tol=1e-10, solver_max_iter=4000,
                               force_reinit=force_reinit))
    P.sync_state(gb, ob)
    return gb, ob


def _gpu_system(gb):
    return {n: gb.download_system(n) for n in
            ("eta_adv", "gamma_adv", "dmass", "w_east", "w_south", "r0", "rhs", "dx")}


def _oracle_system(ob):
    o = ob.copy()
    o.update_maps()
    o.advection()
    A = o.assemble()
    nT, nP = o.p.nTheta, o.p.nPhi
    return A["val"].reshape(nT, nP, 5), A["rhs"].reshape(nT, nP), A["gamma"], o.a["eta"]


def _check_system(S, val, rhs, gamma_adv, eta_adv):
    nT, nP = rhs.shape
    broken_ref = (val[..., 2] == 1.0) & (val[..., 1] == 0.0) & (val[..., 3] == 0.0)
    broken = (S["dmass"] == 1.0) & (S["w_east"] == 0.0) & (S["r0"] == 0.0) & \
        (S["rhs"] == S["gamma_adv"])
    np.testing.assert_array_equal(broken, broken_ref)
    u = ~broken_ref
    assert P.rel_err(S["eta_adv"], eta_adv) <= 1e-5
    assert P.rel_err(S["gamma_adv"][u], gamma_adv[u]) <= 1e-5
    # a broken cell holds gmax (FP32-rounded on the GPU)
    np.testing.assert_allclose(S["gamma_adv"][broken_ref], gamma_adv[broken_ref], rtol=1e-7)
    # couplings: the stored weight between two unbroken cells is the
    # reference's off-diagonal with the sign flipped (both rows hold it)
    wE, wS = S["w_east"], S["w_south"]
    uE = u & np.roll(u, -1, axis=1)  # the east neighbour unbroken too
    uW = u & np.roll(u, 1, axis=1)
    np.testing.assert_allclose(wE[uE], -val[..., 3][uE], rtol=1e-5)
    np.testing.assert_allclose(np.roll(wE, 1, axis=1)[uW], -val[..., 1][uW], rtol=1e-5)
    uS = u[:-1] & u[1:]
    np.testing.assert_allclose(wS[:-1][uS], -val[:-1, :, 4][uS], rtol=1e-5)
    np.testing.assert_allclose(wS[:-1][uS], -val[1:, :, 0][uS], rtol=1e-5)
    assert not wS[-1].any()  # no coupling across the south pole
    # the reference's diagonal
    diag = S["dmass"] + wE + np.roll(wE, 1, axis=1)
    diag[:-1] += wS[:-1]
    diag[1:] += wS[:-1]
    np.testing.assert_allclose(diag[u], val[..., 2][u], rtol=1e-5)
    # b and r0 = b - A gamma_adv (the reference's matrix, FP64)
    bmax = np.max(np.abs(rhs))
    assert np.max(np.abs(S["rhs"][u] - rhs[u])) <= 1e-5 * bmax
    np.testing.assert_allclose(S["rhs"][broken_ref], rhs[broken_ref], rtol=1e-7)
    g = gamma_adv
    Ag = val[..., 2] * g + val[..., 1] * np.roll(g, 1, axis=1) + val[..., 3] * np.roll(g, -1, axis=1)
    Ag[1:] += val[1:, :, 0] * g[:-1]
    Ag[:-1] += val[:-1, :, 4] * g[1:]
    r0_ref = rhs - Ag
    assert np.max(np.abs(S["r0"][u] - r0_ref[u])) <= 1e-5 * bmax


@pytest.mark.parametrize("case", [("c0", 64, 0.005, 4, 1.0, 11, 0), ("c1", 128, 0.002, 6, 0.02, 12, 0),
                                  ("c0", 64, 0.005, 2, 0.5, 13, 2)],
                         ids=lambda c: f"{c[0]}-{c[1]}" + ("-reinit" if c[6] == 2 else ""))
def test_assembled_system_is_the_references_matrix(oracle, gpulib, case):
    """The system stays readable after the step, a step that re-initialises
    the maps included (force_reinit 2: every step)."""
    recipe, nT, dt, pre, t, seed, force = case
    gb, ob = _pair(oracle, recipe, nT, dt, pre, t, seed, force_reinit=force)
    try:
        val, rhs, gamma_adv, eta_adv = _oracle_system(ob)
        gb.step(1, t, dt)
        if force == 2:
            assert gb.stats().reinit == 1
        S = _gpu_system(gb)
        _check_system(S, val, rhs, gamma_adv, eta_adv)
        # the solved increment is the step's change of gamma where nothing
        # clamps (a re-initialisation corrects gamma after the solve)
        if not gb.stats().reinit:
            g_new = gb.download("gamma")
            inner = (S["dmass"] != 1.0) & (g_new > 0) & (g_new < ob.p.gammaMax - 1e-6)
            assert np.max(np.abs(S["gamma_adv"] + S["dx"] - g_new)[inner]) <= 1e-6 * np.max(g_new)
    finally:
        gb.close()


def test_tiny_surfactant_keeps_the_solve_in_range(oracle, gpulib):
    """A patch of 1e-30 surfactant (the FP64 reference's diagonal there is
    1e32 and more) and a patch of 1e-40 (an FP32 subnormal, whose diagonal
    term overflows FP32): their rows are scaled by powers of two, so the
    diagonal stays at most 2^48, the solve converges, the step matches the
    FP64 oracle at the usual tolerance, and the new gamma of every patch
    cell matches the oracle's relative to its own size (1e-3), broken
    status included."""
    nT = 64
    patches = ((slice(20, 26), slice(30, 40), 1e-30), (slice(40, 44), slice(70, 76), 1e-40))

    def patch(ob):
        for r, c, v in patches:
            ob.a["gamma"][r, c] = v

    gb, ob = _pair(oracle, "c0", nT, 0.005, 3, 0.5, 21, gamma_patch=patch)
    try:
        gb.step(1, 0.5, 0.005)
        s = gb.stats()
        assert s.solver_converged == 1 and s.solver_nonconverged == 0
        S = _gpu_system(gb)
        assert np.isfinite(S["dmass"]).all() and S["dmass"].max() <= 2.0 ** 49
        for r, c, v in patches:
            assert S["gamma_adv"][r, c].min() <= 2 * v  # the patches survived advection
        g = gb.download("gamma")
        assert np.isfinite(g).all()
        ob.step()
        for name in ("eta", "gamma", "u_theta", "u_phi"):
            assert P.rel_err(gb.download(name), ob.a[P.FIELD_MAP[name]]) <= 1e-5, name
        gmax = ob.p.gammaMax
        for r, c, v in patches:
            a, b = g[r, c], ob.a["gamma"][r, c]
            np.testing.assert_array_equal(a > 0.5 * gmax, b > 0.5 * gmax)
            small = b < 0.5 * gmax
            np.testing.assert_allclose(a[small], b[small], rtol=1e-3, atol=0)
    finally:
        gb.close()


def test_cells_at_the_fp32_gmax_are_broken(gpulib):
    """The reference marks gamma > gmax - 1e-7 as at the maximum
    (kernel/bubble.cu:1317).  At gmax ~ 29 that band is below FP32's
    resolution and gmax - 1e-7 rounds to gmax itself, so a threshold taken
    literally in FP32 would leave cells holding gmax (every clamped cell)
    unbroken, and a broken cell that the assembly sets to gmax would look
    unbroken to a neighbour reading it afterwards.  Cells whose advected
    concentration is the FP32 gmax must get the identity row."""
    from soapbubble_gb300 import synth
    from soapbubble_gb300.bubble import GpuBubble, make_params
    nT = 64
    f = synth.make_fields("c0", nT, 31)
    gb = GpuBubble(make_params(nT, 0.005))
    try:
        gb.upload_fields(f.eta, f.gamma, f.uth, f.uph, f.uair_init, f.vair_init)
        gmax32 = float(np.float32(29.347029))  # the default parameters' gmax in FP32
        g = gb.download("gamma")
        g[20:30, 40:60] = gmax32
        gb.upload("gamma", g)
        gb.step(1, 0.0, 0.005)
        S = _gpu_system(gb)
        inner = (slice(22, 28), slice(42, 58))  # stencils inside the patch
        assert np.all(S["dmass"][inner] == 1.0) and not S["w_east"][inner].any()
        assert np.all(S["r0"][inner] == 0.0)
        assert gb.stats().broken_cells >= 6 * 16
    finally:
        gb.close()


@pytest.mark.parametrize("mode", [0, 1], ids=["mixed", "plain"])
def test_twin_bubbles_stay_identical_through_the_rupture(gpulib, mode):
    """Two bubbles from the same fields, stepped on their own streams so that
    their kernels overlap, through the film's rupture (broken cells from
    about step 300 at this grid): bit-identical fields at the end, with the
    mixed-precision and the plain FP32 solve (both warm-started).  A read of
    a value that another thread of the same kernel writes would make the
    twins differ."""
    from soapbubble_gb300 import synth
    from soapbubble_gb300.bubble import GpuBubble, make_params
    nT, dt = 128, 0.002
    f = synth.make_fields("c1", nT, 20261203)
    a = GpuBubble(make_params(nT, dt, solver_tol=1e-6, solver_mode=mode))
    b = GpuBubble(make_params(nT, dt, solver_tol=1e-6, solver_mode=mode))
    try:
        for gb in (a, b):
            gb.upload_fields(f.eta, f.gamma, f.uth, f.uph, f.uair_init, f.vair_init)
        broken = 0
        for k in range(0, 600, 10):
            t = k * dt
            a.step(10, t, dt)
            b.step(10, t, dt)
            if k % 100 == 90:
                broken = max(broken, a.stats().broken_cells)
        assert broken > 0  # the run went through the rupture
        for name in ("eta", "gamma", "u_theta", "u_phi", "eta_delta", "gamma_delta", "fwd_t", "bwd_t"):
            np.testing.assert_array_equal(a.download(name), b.download(name), err_msg=name)
    finally:
        a.close()
        b.close()
