"""GPU checks of the runtime around the kernels: graph replay, the frame
loop and its EXR frames, statistics, mass bookkeeping, larger grids."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _bubble(nT, recipe="c0", dt=0.005, seed=3, **kw):
    from soapbubble_gb300 import synth
    from soapbubble_gb300.bubble import GpuBubble, make_params
    f = synth.make_fields(recipe, nT, seed)
    gb = GpuBubble(make_params(nT, dt, **kw))
    gb.upload_fields(f.eta, f.gamma, f.uth, f.uph, f.uair_init, f.vair_init)
    return gb


def test_graph_replay_matches_kernel_by_kernel(gpulib):
    """sb_step (captured CUDA graphs) and sb_step_timed (one launch per
    kernel) run the same kernels: results are bit-identical, also across a
    forced re-initialisation."""
    a = _bubble(64, force_reinit=0)
    b = _bubble(64, force_reinit=0)
    with a, b:
        ms = np.zeros(16)
        for k in range(12):
            t = (k // 10) * 0.05
            a.step(1, t, 0.005)
            b.step_timed(1, t, 0.005, ms)
        for name in ("eta", "gamma", "u_theta", "u_phi", "eta_delta", "fwd_t", "bwd_p"):
            np.testing.assert_array_equal(a.download(name), b.download(name), err_msg=name)
        sa, sb = a.stats(), b.stats()
        assert sa.reinits == sb.reinits and sa.steps == sb.steps == 12
        assert sa.launches == sb.launches
        assert ms.sum() > 0


def test_frame_loop_writes_reference_frames(gpulib, tmp_path):
    """sb_run: frame0000.exr .. frame0003.exr, 3 equal HALF channels of
    eta * H * 2e5 (kernel/solver.cu:541-593)."""
    from soapbubble_gb300.exr import read_exr
    gb = _bubble(32, dt=0.005, DT=0.02, frames=4)
    with gb:
        gb.run(str(tmp_path) + "/", frames=4)
        names = sorted(os.listdir(tmp_path))
        assert names == [f"frame{i:04d}.exr" for i in range(4)]
        last = read_exr(str(tmp_path / "frame0003.exr"))
        eta = gb.download("eta").astype(np.float32)
        expect = (eta.astype(np.float64) * 1e-6 * 2e5).astype(np.float32).astype(np.float16)
        for c in "BGR":
            np.testing.assert_array_equal(last[c], expect.astype(np.float32))
        # 3 frames of 4 steps each
        assert gb.stats().steps == 12


def _velocity_image(uth, uph):
    """Solver::write_velocity_image (kernel/solver.cu:388-497) in numpy."""
    uth, uph = uth.astype(np.float64), uph.astype(np.float64)
    nT, nP = uph.shape
    opp = (np.arange(nP) + nP // 2) % nP
    u = 0.5 * (uph + np.roll(uph, -1, axis=1))
    vN = np.vstack([0.75 * uth[:1] - 0.25 * uth[:1, opp], uth])
    vS = np.vstack([uth, 0.75 * uth[-1:] - 0.25 * uth[-1:, opp]])
    v = 0.5 * (vN + vS)
    return (u / 2 + 0.5).astype(np.float32), (v / 2 + 0.5).astype(np.float32)


def test_velocity_and_concentration_frames(gpulib, tmp_path):
    """vel%04d.exr (R = u/2 + 0.5, G = v/2 + 0.5, B = 0.5) and con%04d.exr
    ((gamma - 0.9) / 0.2 in all channels) beside the thickness frames when
    the params ask for them (WRITE_VELOCITY_DATA, WRITE_CONCENTRATION_DATA)."""
    from soapbubble_gb300.exr import read_exr
    gb = _bubble(32, dt=0.005, DT=0.01, frames=3, write_velocity_frames=1,
                 write_concentration_frames=1)
    with gb:
        gb.run(str(tmp_path) + "/", frames=3)
        names = sorted(os.listdir(tmp_path))
        assert names == sorted([f"{k}{i:04d}.exr" for k in ("frame", "vel", "con")
                                for i in range(3)])
        R, G = _velocity_image(gb.download("u_theta"), gb.download("u_phi"))
        vel = read_exr(str(tmp_path / "vel0002.exr"))
        np.testing.assert_array_equal(vel["R"], R.astype(np.float16).astype(np.float32))
        np.testing.assert_array_equal(vel["G"], G.astype(np.float16).astype(np.float32))
        assert np.all(vel["B"] == 0.5)
        assert np.abs(vel["R"] - 0.5).max() > 1e-3  # the wind moved the film
        con = read_exr(str(tmp_path / "con0002.exr"))
        gam = gb.download("gamma").astype(np.float32).astype(np.float64)
        expect = ((gam - 0.9) / 0.2).astype(np.float32).astype(np.float16).astype(np.float32)
        for c in "BGR":
            np.testing.assert_array_equal(con[c], expect)
        # the writers also work on their own
        gb.write_velocity_exr(str(tmp_path / "v.exr"))
        gb.write_concentration_exr(str(tmp_path / "c.exr"))
        np.testing.assert_array_equal(read_exr(str(tmp_path / "v.exr"))["G"], vel["G"])


def test_stats_and_mass_bookkeeping(gpulib):
    gb = _bubble(64)
    with gb:
        s0 = gb.stats(mass=True)
        nT, nP = 64, 128
        eta = gb.download("eta")
        # the GPU's sin table is FP64 rounded to FP32
        s = np.sin((np.arange(nT) + 0.5) * np.pi / nT).astype(np.float32).astype(np.float64)[:, None]
        assert s0.mass_eta == pytest.approx(float((eta * s).sum()), rel=1e-12)
        gb.step(5, 0.0, 0.005)
        s1 = gb.stats(mass=True)
        assert s1.steps == 5 and s1.solver_converged == 1
        assert 0 < s1.solver_iters < 50 and s1.solver_rel_resid <= 1e-6
        # evaporation thins the film a little each step
        assert s1.mass_eta < s0.mass_eta


@pytest.mark.parametrize("nT,recipe,dt", [(512, "c1", 0.002), (1024, "c2", 0.001)])
def test_full_size_steps_are_sane(gpulib, nT, recipe, dt):
    """The benchmark grids: 20 steps stay finite, the solve converges to
    1e-6 every step, the film stays non-negative, mass drifts only slowly."""
    gb = _bubble(nT, recipe, dt, seed=9)
    with gb:
        m0 = gb.stats(mass=True).mass_eta
        for k in range(20):
            gb.step(1, (k // 10) * 10 * dt, dt)
            s = gb.stats()
            assert s.solver_converged == 1 and s.solver_rel_resid <= 1e-6
        s = gb.stats(mass=True)
        eta = gb.download("eta")
        assert np.isfinite(eta).all() and eta.min() >= 0.0
        for name in ("gamma", "u_theta", "u_phi"):
            assert np.isfinite(gb.download(name)).all(), name
        assert abs(s.mass_eta - m0) / m0 < 0.05


def test_autotuned_tiles_give_identical_results(gpulib):
    """sb_autotune only changes how many cells a block covers: a tuned
    bubble and an untuned twin stay bit-identical."""
    a = _bubble(64, force_reinit=0)
    b = _bubble(64, force_reinit=0)
    with a, b:
        tiles = a.autotune(0.0, 0.005)
        ms = np.zeros(16)
        b.step_timed(3, 0.0, 0.005, ms)
        assert all(t in (64, 128, 256) for t in tiles[:8])
        for k in range(10):
            a.step(1, 0.0, 0.005)
            b.step(1, 0.0, 0.005)
        for name in ("eta", "gamma", "u_theta", "u_phi", "eta_delta", "fwd_t", "bwd_p"):
            np.testing.assert_array_equal(a.download(name), b.download(name), err_msg=name)
        assert a.stats().steps == b.stats().steps == 13


@pytest.mark.parametrize("storage", [0, 1], ids=["fp32", "bf16"])
def test_staged_io_matches_synchronous_io(gpulib, storage):
    """Forcing uploaded and thickness read back through the copy stream
    (sb_stage_*) give the same steps, bit for bit, as the synchronous
    copies; each step's staged download holds that step's field."""
    from soapbubble_gb300 import cudart
    from soapbubble_gb300._lib import SB_ERR_INVALID, SoapBubbleError
    nT = 64
    a = _bubble(nT, storage=storage)
    b = _bubble(nT, storage=storage)
    N, Nv = nT * 2 * nT, (nT - 1) * 2 * nT
    rng = np.random.default_rng(9)
    winds = [(rng.uniform(-1, 1, N).astype(np.float32), rng.uniform(-1, 1, Nv).astype(np.float32))
             for _ in range(6)]
    hu = [cudart.PinnedArray((N,)) for _ in range(2)]
    hv = [cudart.PinnedArray((Nv,)) for _ in range(2)]
    he = [cudart.PinnedArray((N,)) for _ in range(6)]
    try:
        with a, b:
            for k, (u, v) in enumerate(winds):
                a.upload_f32("uair_init", u)
                a.upload_f32("vair_init", v)
                a.step(1, 0.0, 0.005)
                want = a.download("eta").astype(np.float32).ravel()
                hu[k & 1].array[:] = u
                hv[k & 1].array[:] = v
                if k >= 2:
                    b.wait_staged()  # the pinned inputs of step k - 2 are free again
                b.stage_upload_f32("uair_init", hu[k & 1].array)
                b.stage_upload_f32("vair_init", hv[k & 1].array)
                if k == 0:
                    with pytest.raises(SoapBubbleError) as e:
                        b.stage_upload_f32("vair_init", hv[0].array)
                    assert e.value.code == SB_ERR_INVALID
                b.step(1, 0.0, 0.005)
                b.stage_download_f32("eta", he[k].array)
                b.wait_staged()
                np.testing.assert_array_equal(he[k].array, want, err_msg=f"step {k}")
            for name in ("eta", "gamma", "u_theta", "u_phi", "uair_init", "vair_init"):
                np.testing.assert_array_equal(a.download(name), b.download(name), err_msg=name)
            # a staged download of a field written by an upload in flight sees the upload
            b.stage_upload_f32("uair_init", hu[0].array)
            b.step(1, 0.0, 0.005)
            out = cudart.PinnedArray((N,))
            b.stage_download_f32("uair_init", out.array)
            b.wait_staged()
            np.testing.assert_array_equal(out.array, hu[0].array)
            out.free()
    finally:
        for h in hu + hv + he:
            h.free()
