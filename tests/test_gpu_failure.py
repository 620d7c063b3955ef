"""Failure reporting on the GPU, made without any GPU fault.

A solve that misses its tolerance is made by asking for more than one PCG
iteration can give (tolerance 1e-12, iteration limit 1): it must show in the
statistics (solver_converged, the running non-converged count and worst
residual), in sb_synchronize's status, and it must stop sb_run right after
its step, as the reference's AmgX failure stops Bubble::run
(kernel/bubble.cu:1500-1507, 2669-2682).  A grid barrier whose wait runs
out is made with the library's self-test, in which one block of four never
arrives and the others give up after a short poll limit (a bounded wait
that returns an error status; no block waits without a limit)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIELDS = ("eta", "gamma", "u_theta", "u_phi", "fwd_t", "bwd_p", "eta_delta")


def _bubble(nT=64, seed=5, **kw):
    from soapbubble_gb300 import synth
    from soapbubble_gb300.bubble import GpuBubble, make_params
    f = synth.make_fields("c0", nT, seed)
    gb = GpuBubble(make_params(nT, 0.005, **kw))
    gb.upload_fields(f.eta, f.gamma, f.uth, f.uph, f.uair_init, f.vair_init)
    return gb


def _raw_stats(gb):
    """sb_get_stats without raising (it fills the stats on error too)."""
    import ctypes as C
    from soapbubble_gb300._lib import SbStats, lib
    s = SbStats()
    rc = lib().sb_get_stats(gb.h, C.byref(s))
    return rc, s


def test_nonconverged_solve_is_counted_and_reported(gpulib):
    from soapbubble_gb300._lib import SB_ERR_NOT_CONVERGED, SoapBubbleError
    with _bubble(solver_tol=1e-12, solver_max_iter=1) as gb:
        gb.synchronize()  # no solve yet: nothing to report
        gb.step(1, 0.0, 0.005)
        with pytest.raises(SoapBubbleError) as e:
            gb.synchronize()
        assert e.value.code == SB_ERR_NOT_CONVERGED
        s = gb.stats()
        assert s.solver_converged == 0 and s.solver_iters == 1
        assert s.solves == 1 and s.solver_nonconverged == 1
        assert s.solver_rel_resid_max > 1e-12 and s.solver_rel_resid_max == s.solver_rel_resid
        gb.step(2, 0.0, 0.005)
        s = gb.stats()
        assert s.solves == 3 and s.solver_nonconverged == 3 and s.steps == 3
        gb.reset_stats()
        s = gb.stats()
        assert s.solver_nonconverged == 0 and s.solver_rel_resid_max == 0.0 and s.solves == 3
    # the same bubble with a reachable target: converged, nothing counted
    with _bubble(solver_tol=1e-6) as gb:
        gb.step(3, 0.0, 0.005)
        gb.synchronize()
        s = gb.stats()
        assert s.solver_converged == 1 and s.solver_nonconverged == 0 and s.solves == 3
        assert 0.0 < s.solver_rel_resid_max <= 1e-6


def test_run_stops_right_after_the_failing_step(gpulib):
    """sb_run with frames of 4 steps: the first solve fails, so the run
    returns SB_ERR_NOT_CONVERGED after one step (the device skips the
    frame's other three), the state equals one sb_step of a twin, and the
    bubble steps normally again afterwards."""
    from soapbubble_gb300._lib import SB_ERR_NOT_CONVERGED, SoapBubbleError
    kw = dict(solver_tol=1e-12, solver_max_iter=1, DT=0.02, frames=3)
    with _bubble(**kw) as a, _bubble(**kw) as b:
        with pytest.raises(SoapBubbleError) as e:
            a.run(None, frames=3)
        assert e.value.code == SB_ERR_NOT_CONVERGED
        assert a.stats().steps == 1
        b.step(1, 0.0, 0.005)
        for name in FIELDS:
            np.testing.assert_array_equal(a.download(name), b.download(name), err_msg=name)
        # the halt ends with the run: both step on identically
        a.step(2, 0.02, 0.005)
        b.step(2, 0.02, 0.005)
        assert a.stats().steps == 3
        for name in FIELDS:
            np.testing.assert_array_equal(a.download(name), b.download(name), err_msg=name)


def test_run_without_failure_takes_every_step(gpulib):
    with _bubble(DT=0.02, frames=3) as gb:
        gb.run(None, frames=3)
        s = gb.stats()
        assert s.steps == 8 and s.solver_nonconverged == 0 and s.solves == 8


def test_grid_barrier_wait_gives_up_and_reports(gpulib):
    """Self-test of the bounded grid barrier: with every block arriving
    nothing is counted; with block 2 of 4 absent the other three give up
    after 2^16 polls, sb_get_stats returns SB_ERR_CUDA, and the bubble halts
    at the end of its next step (its fields stop changing)."""
    from soapbubble_gb300._lib import SB_ERR_CUDA, SB_OK, lib
    L = lib()
    with _bubble() as gb:
        gb.step(1, 0.0, 0.005)
        assert L.sb_selftest_grid_barrier(gb.h, -1, 1 << 16) == SB_OK
        assert _raw_stats(gb)[0] == SB_OK
        gb.step(1, 0.0, 0.005)  # the barrier word still works for the solve
        assert _raw_stats(gb)[1].solver_converged == 1
        assert L.sb_selftest_grid_barrier(gb.h, 2, 1 << 16) == SB_OK
        rc, s = _raw_stats(gb)
        assert rc == SB_ERR_CUDA
        assert b"bounded wait" in L.sb_last_error()
        assert L.sb_step(gb.h, 1, 0.0, 0.005) == SB_OK  # halts at its end
        rc, s = _raw_stats(gb)
        assert rc == SB_ERR_CUDA and s.steps == 3
        before = {n: gb.download(n) for n in FIELDS}
        assert L.sb_step(gb.h, 2, 0.0, 0.005) == SB_OK
        rc, s = _raw_stats(gb)
        assert s.steps == 3
        for n in FIELDS:
            np.testing.assert_array_equal(gb.download(n), before[n], err_msg=n)
    with _bubble() as gb:
        assert L.sb_selftest_grid_barrier(gb.h, 4, 1 << 16) != SB_OK  # no block 4
        assert L.sb_selftest_grid_barrier(gb.h, 0, 0) != SB_OK        # no zero limit
        assert _raw_stats(gb)[0] == SB_OK
