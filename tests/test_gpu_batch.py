"""GPU checks of the batched ensemble (sb_batch_*): many bubbles of uneven
grid size and coefficients stepped by one launch per stage.

Every batched kernel runs the same per-cell arithmetic as the single-bubble
kernels, and the implicit solve sums each system's dot products row by row
in row order whatever the block distribution, so a member stepped inside a
batch matches the same bubble stepped alone bit for bit.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIELDS = ("eta", "gamma", "u_theta", "u_phi", "eta_delta", "gamma_delta", "eta_init",
          "gamma_init", "eta_delta_last", "fwd_t", "fwd_p", "bwd_t", "bwd_p", "bwdprev_t")


def _member(nT, seed, recipe="c0", dt=0.005, scales=(1.0, 1.0, 1.0), **kw):
    from soapbubble_gb300 import synth
    from soapbubble_gb300.bubble import GpuBubble, make_params
    f = synth.make_fields(recipe, nT, seed)
    gs, nu, M = scales
    gb = GpuBubble(make_params(nT, dt, gs_scale=gs, nu_scale=nu, M_scale=M, **kw))
    gb.upload_fields(f.eta, f.gamma, f.uth, f.uph, f.uair_init, f.vair_init)
    return gb


def _twins(specs, **kw):
    """Two identical sets of bubbles: one for the batch, one stepped alone."""
    a = [_member(*s, **kw) for s in specs]
    b = [_member(*s, **kw) for s in specs]
    return a, b


def _schedule(nsteps, dt):
    # the frame time changes every 5 steps, as in the frame loop
    return [((k // 5) * 5 * dt, dt) for k in range(nsteps)]


def _close(bubbles):
    for g in bubbles:
        g.close()


SMALL = [(16, 11, "c0", 0.005, (1.4, 0.7, 1.2)),
         (32, 12, "c0", 0.005, (0.6, 1.3, 0.8)),
         (64, 13, "c1", 0.005, (1.0, 1.0, 1.0)),
         (8, 14, "c0", 0.005, (1.2, 1.2, 0.5))]


@pytest.mark.parametrize("solver_mode", [0, 1], ids=["mixed", "plain"])
def test_batch_matches_members_stepped_alone(gpulib, solver_mode):
    from soapbubble_gb300.bubble import GpuBatch
    a, b = _twins(SMALL, solver_mode=solver_mode, solver_tol=1e-6)
    try:
        with GpuBatch(a) as batch:
            for t, dt in _schedule(25, 0.005):
                batch.step(1, t, dt)
                for g in b:
                    g.step(1, t, dt)
            batch.synchronize()
        for ga, gb in zip(a, b):
            for name in FIELDS:
                np.testing.assert_array_equal(ga.download(name), gb.download(name),
                                              err_msg=f"nT={ga.nTheta} {name}")
            sa, sb = ga.stats(), gb.stats()
            assert sa.steps == sb.steps == 25
            assert sa.reinits == sb.reinits
            assert sa.solver_iters == sb.solver_iters
            assert sa.solver_rel_resid == sb.solver_rel_resid
            assert sa.solver_converged == sb.solver_converged == 1
            assert sa.distortion == sb.distortion
    finally:
        _close(a + b)


def test_batch_reinit_decided_per_member(gpulib):
    """One member re-initialises every step (forced), the others never or by
    their own distortion: each follows its own decision inside the shared
    cooperative launch."""
    from soapbubble_gb300.bubble import GpuBatch
    specs = [(16, 21), (32, 22), (32, 23)]
    forces = [2, 1, 0]
    a = [_member(*s, force_reinit=f) for s, f in zip(specs, forces)]
    b = [_member(*s, force_reinit=f) for s, f in zip(specs, forces)]
    try:
        with GpuBatch(a) as batch:
            for t, dt in _schedule(12, 0.005):
                batch.step(1, t, dt)
                for g in b:
                    g.step(1, t, dt)
            batch.synchronize()
        reinits = [g.stats().reinits for g in a]
        assert reinits[0] == 12 and reinits[1] == 0
        for ga, gb in zip(a, b):
            assert ga.stats().reinits == gb.stats().reinits
            for name in FIELDS:
                np.testing.assert_array_equal(ga.download(name), gb.download(name), err_msg=name)
    finally:
        _close(a + b)


def test_batch_timed_autotuned_and_graph_paths_agree(gpulib):
    """The stage-by-stage path, the autotuner's tuning steps (every tile
    size) and the captured graph with the tuned tiles give the results of
    stepping the members alone."""
    from soapbubble_gb300.bubble import GpuBatch, stage_names
    a, b = _twins(SMALL[:3])
    try:
        with GpuBatch(a) as batch:
            ms = np.zeros(16)
            batch.step_timed(2, 0.0, 0.005, ms)
            tiles = batch.autotune(0.0, 0.005)
            batch.step(3, 0.025, 0.005)
            batch.synchronize()
            assert ms[:len(stage_names())].sum() > 0
            assert all(t in (64, 128, 256) for t in tiles[:len(stage_names())])
        for g in b:
            g.step(5, 0.0, 0.005)
            g.step(3, 0.025, 0.005)
        for ga, gb in zip(a, b):
            assert ga.stats().steps == gb.stats().steps == 8
            for name in FIELDS:
                np.testing.assert_array_equal(ga.download(name), gb.download(name), err_msg=name)
    finally:
        _close(a + b)


def test_ensemble_matches_members_stepped_alone(gpulib):
    """The 64-bubble ensemble (nTheta 64..512, seeded coefficients): a few
    batched steps against each member stepped alone, bit for bit."""
    from soapbubble_gb300 import synth
    from soapbubble_gb300.bubble import GpuBatch
    dt = synth.ENSEMBLE["dt"]
    members = synth.ensemble(seed=4)
    specs = [(m.nTheta, m.seed, "c0", dt, (m.gs_scale, m.nu_scale, m.M_scale)) for m in members]
    a, b = _twins(specs)
    try:
        with GpuBatch(a) as batch:
            for t, d in _schedule(6, dt):
                batch.step(1, t, d)
                for g in b:
                    g.step(1, t, d)
            batch.synchronize()
        for ga, gb in zip(a, b):
            sa, sb = ga.stats(), gb.stats()
            assert sa.solver_converged == 1 and sa.solver_rel_resid <= 1e-6
            assert sa.steps == sb.steps == 6
            assert sa.solver_iters == sb.solver_iters and sa.reinits == sb.reinits
            for name in ("eta", "gamma", "u_theta", "u_phi", "eta_delta", "fwd_t", "bwd_p"):
                np.testing.assert_array_equal(ga.download(name), gb.download(name),
                                              err_msg=f"nT={ga.nTheta} {name}")
    finally:
        _close(a + b)


def test_batch_rejects_mixed_solver_settings(gpulib):
    from soapbubble_gb300._lib import SoapBubbleError
    from soapbubble_gb300.bubble import GpuBatch
    a = _member(16, 1, solver_mode=0)
    b = _member(16, 2, solver_mode=1)
    try:
        with pytest.raises(SoapBubbleError, match="solver"):
            GpuBatch([a, b])
    finally:
        _close([a, b])


def test_viscous_batch_matches_members_stepped_alone(gpulib):
    from soapbubble_gb300.bubble import GpuBatch
    a, b = _twins(SMALL[:3], viscous=1, radius=0.05, solver_tol=1e-6)
    try:
        with GpuBatch(a) as batch:
            for t, dt in _schedule(10, 0.005):
                batch.step(1, t, dt)
                for g in b:
                    g.step(1, t, dt)
            batch.synchronize()
        for ga, gb in zip(a, b):
            for name in FIELDS:
                np.testing.assert_array_equal(ga.download(name), gb.download(name),
                                              err_msg=f"nT={ga.nTheta} {name}")
    finally:
        _close(a + b)


def test_batch_rejects_mixed_viscous_switch(gpulib):
    from soapbubble_gb300._lib import SoapBubbleError
    from soapbubble_gb300.bubble import GpuBatch
    a = _member(16, 1, viscous=0)
    b = _member(16, 2, viscous=1)
    try:
        with pytest.raises(SoapBubbleError, match="viscous"):
            GpuBatch([a, b])
    finally:
        _close([a, b])


def test_wide_rows_batch_matches_members_stepped_alone(gpulib):
    """A set whose widest rows have 2048 columns runs the solve with
    512-thread blocks; its smaller members still match themselves stepped
    alone (256-thread blocks) bit for bit: the dot products are formed in an
    order that does not depend on the block width."""
    from soapbubble_gb300.bubble import GpuBatch
    specs = [(1024, 21, "c2", 0.001, (1.0, 1.0, 1.0)), (64, 22, "c0", 0.001, (1.2, 0.8, 1.1)),
             (256, 23, "c1", 0.001, (0.9, 1.1, 1.0)), (512, 24, "c1", 0.001, (1.0, 1.0, 1.0))]
    a, b = _twins(specs, solver_tol=1e-6)
    try:
        with GpuBatch(a) as batch:
            for t, dt in _schedule(4, 0.001):
                batch.step(1, t, dt)
                for g in b:
                    g.step(1, t, dt)
            batch.synchronize()
        for ga, gb in zip(a, b):
            for name in ("eta", "gamma", "u_theta", "u_phi", "eta_delta", "fwd_t"):
                np.testing.assert_array_equal(ga.download(name), gb.download(name),
                                              err_msg=f"nT={ga.nTheta} {name}")
            assert ga.stats().solver_iters == gb.stats().solver_iters
    finally:
        _close(a + b)


def test_retired_member_is_left_untouched(gpulib):
    """sb_batch_retire: a member retired after 6 steps keeps its state while
    the batch steps on, and the other members still match the same bubbles
    stepped alone bit for bit (the retired member's rows leave the solve,
    whose exact sums do not depend on which rows take part)."""
    from soapbubble_gb300.bubble import GpuBatch
    a, b = _twins(SMALL[:3], solver_tol=1e-6)
    try:
        with GpuBatch(a) as batch:
            for k, (t, dt) in enumerate(_schedule(15, 0.005)):
                if k == 6:
                    batch.synchronize()
                    kept = {n: a[1].download(n) for n in FIELDS}
                    batch.retire(1)
                batch.step(1, t, dt)
                for i, g in enumerate(b):
                    if i != 1 or k < 6:
                        g.step(1, t, dt)
            batch.synchronize()
        for n in FIELDS:
            np.testing.assert_array_equal(a[1].download(n), kept[n], err_msg=n)
            for i in (0, 2):
                np.testing.assert_array_equal(a[i].download(n), b[i].download(n), err_msg=n)
        assert a[1].stats().steps == 6 and a[0].stats().steps == 15
    finally:
        _close(a + b)
