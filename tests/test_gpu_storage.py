"""GPU checks of the BF16 storage of the thickness and surfactant fields
(SB_STORE_BF16: eta, gamma and the BIMOCQ reference fields in BF16 between
steps, the BIMOCQ change accumulators in FP32, FP32 arithmetic).

A BF16 field holds the deviation from a per-field base (the BF16-rounded
mean at upload), so it keeps 8 significant bits of the deviation, not of
the value.  The storage variant is compared against the FP64 oracle at that
precision, not at the 1e-5 of the FP32 path: after one step from identical
inputs every stored field carries at most one BF16 rounding of its
deviation (plus FP32 noise).
"""
import numpy as np
import pytest

import _parity as P

pytestmark = pytest.mark.gpu

U_BF16 = 2.0 ** -8   # BF16 spacing relative to the value (rounding error <= half of it)


def bf16_round(x):
    """Round FP32 values to BF16 (nearest, ties to even), returned as FP32."""
    a = np.asarray(x, dtype=np.float32).copy()
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) >> 16 << 16
    return u.astype(np.uint32).view(np.float32)


def _bubble(nT, recipe, seed, storage, **kw):
    from soapbubble_gb300 import synth
    from soapbubble_gb300.bubble import GpuBubble, make_params
    dt = {"c0": 0.005, "c1": 0.002, "c2": 0.001}[recipe]
    f = synth.make_fields(recipe, nT, seed)
    gb = GpuBubble(make_params(nT, dt, storage=storage, **kw))
    gb.upload_fields(f.eta, f.gamma, f.uth, f.uph, f.uair_init, f.vair_init)
    gb.fields = f
    return gb, dt


def stored(v, base):
    """What a BF16 field holds for FP32 values v with offset `base`:
    base + bf16(v - base), in FP32 arithmetic."""
    v = np.asarray(v, dtype=np.float32)
    return (bf16_round(v - np.float32(base)) + np.float32(base)).astype(np.float32)


def test_bf16_fields_round_trip_and_memory(gpulib):
    from soapbubble_gb300.bubble import bytes_required, make_params
    gb, _ = _bubble(64, "c0", 3, 1)
    try:
        # the offsets are the BF16-rounded means of the uploaded fields
        base_g = bf16_round(np.float32(np.mean(gb.fields.gamma)))
        base_e = bf16_round(np.float32(np.mean(gb.fields.eta)))
        x = np.random.default_rng(0).uniform(0.9, 1.1, gb.nTheta * gb.nPhi)
        gb.upload("gamma_init", x)
        np.testing.assert_array_equal(gb.download("gamma_init").ravel(),
                                      stored(x, base_g).astype(np.float64))
        # the FP32 entry points convert on the device too
        y = np.random.default_rng(1).uniform(0.8, 1.2, gb.nTheta * gb.nPhi).astype(np.float32)
        gb.upload_f32("eta", y)
        out = np.zeros_like(y)
        gb.download_f32("eta", out)
        gb.synchronize()
        np.testing.assert_array_equal(out, stored(y, base_e))
        # a vanished film stays exactly zero
        z = np.zeros_like(y)
        gb.upload_f32("eta", z)
        gb.download_f32("eta", out)
        gb.synchronize()
        assert not out.any()
    finally:
        gb.close()
    # six fields of nTheta x nPhi elements shrink from 4 to 2 bytes
    n = 256 * 512
    saved = bytes_required(make_params(256, 0.005)) - bytes_required(make_params(256, 0.005,
                                                                                 storage=1))
    assert saved >= 6 * n * 2 - 6 * 256 and saved <= 6 * n * 2 + 6 * 256, saved


@pytest.mark.parametrize("case", [("c0", 64, 0.005, 5, 1.0, 1234), ("c2", 128, 0.001, 5, 0.5, 78)],
                         ids=lambda c: f"{c[0]}-{c[1]}")
def test_bf16_step_matches_oracle_at_bf16_precision(oracle, gpulib, case):
    """One step from identical (BF16-representable) state: thickness and
    surfactant within a BF16 rounding of the FP64 oracle, velocities close."""
    from soapbubble_gb300 import synth
    from soapbubble_gb300.bubble import GpuBubble, make_params
    recipe, nT, dt, pre, t, seed = case
    f = synth.make_fields(recipe, nT, seed)
    op = oracle.default_params(nT, dt_s=dt)
    op.t = t
    ob = oracle.OracleBubble(op, f.eta, f.gamma, f.uth, f.uph, f.uair_init, f.vair_init)
    for _ in range(pre):
        ob.step()
    gb = GpuBubble(make_params(nT, dt, solver_tol=1e-10, solver_max_iter=2000, storage=1))
    try:
        P.sync_state(gb, ob)  # the oracle continues from the BF16-rounded state
        gb.step(1, t, dt)
        ob.step()
        err = P.compare(gb, ob, ["eta", "gamma", "u_theta", "u_phi"])
        assert err["eta"] <= U_BF16, err
        assert err["gamma"] <= U_BF16, err
        assert err["u_theta"] <= 1e-2 and err["u_phi"] <= 1e-2, err
        assert gb.stats().solver_converged == 1
    finally:
        gb.close()


def test_bf16_run_stays_near_fp32(gpulib):
    """Twenty steps in each storage: the BF16 run stays finite, converges,
    and tracks the FP32 run (thickness and surfactant within 1 %)."""
    a, dt = _bubble(64, "c0", 9, 0)
    b, _ = _bubble(64, "c0", 9, 1)
    try:
        for k in range(20):
            a.step(1, (k // 10) * 10 * dt, dt)
            b.step(1, (k // 10) * 10 * dt, dt)
        for name in ("eta", "gamma", "u_theta", "u_phi"):
            assert np.isfinite(b.download(name)).all(), name
        for name in ("eta", "gamma"):
            x, y = a.download(name), b.download(name)
            assert P.rel_err(y, x) <= 1e-2, (name, P.rel_err(y, x))
        assert b.stats().solver_converged == 1
    finally:
        a.close()
        b.close()


def test_bf16_drift_over_the_c2_run_is_the_flows_sensitivity(gpulib):
    """Config c2 (1024 x 2048, dt 0.001 s), 100 steps.  The c2 flow
    amplifies any perturbation of its initial thickness about seventyfold
    over 100 steps: an FP32 run started from the BF16-rounded initial
    fields (4e-4 from the exact ones) ends 2.9e-2 from the FP32 run.  BF16
    storage, which also rounds every step, ends 5.6e-2 away (measured on a
    GB300).  The bound: the BF16 run stays within 3x the drift that the
    initial rounding alone causes, and within 0.1 of the FP32 thickness."""
    from soapbubble_gb300 import synth
    from soapbubble_gb300.bubble import GpuBubble, make_params
    nT, dt = 1024, 0.001
    f = synth.make_fields("c2", nT, 20261203)

    def run(storage, eta, gamma):
        gb = GpuBubble(make_params(nT, dt, solver_tol=1e-6, storage=storage))
        try:
            gb.upload_fields(eta, gamma, f.uth, f.uph, f.uair_init, f.vair_init)
            init = (gb.download("eta"), gb.download("gamma"))
            for k in range(100):
                gb.step(1, (k // 10) * 10 * dt, dt)
            return gb.download("eta"), init
        finally:
            gb.close()

    fp32, _ = run(0, f.eta, f.gamma)
    bf16, (e0, g0) = run(1, f.eta, f.gamma)
    fp32_rounded_start, _ = run(0, e0, g0)
    d_bf16 = P.rel_err(bf16, fp32)
    d_start = P.rel_err(fp32_rounded_start, fp32)
    assert np.isfinite(bf16).all()
    assert d_bf16 <= 3.0 * d_start and d_bf16 <= 0.1, (d_bf16, d_start)


def test_bf16_batch_matches_members_stepped_alone(gpulib):
    from soapbubble_gb300.bubble import GpuBatch
    specs = [(32, "c0", 41), (64, "c0", 42), (16, "c0", 43)]
    a = [_bubble(*s, 1)[0] for s in specs]
    b = [_bubble(*s, 1)[0] for s in specs]
    try:
        with GpuBatch(a) as batch:
            for k in range(12):
                batch.step(1, (k // 5) * 5 * 0.005, 0.005)
                for g in b:
                    g.step(1, (k // 5) * 5 * 0.005, 0.005)
            batch.synchronize()
        for ga, gb in zip(a, b):
            for name in ("eta", "gamma", "u_theta", "u_phi", "eta_delta", "gamma_init", "bwd_t"):
                np.testing.assert_array_equal(ga.download(name), gb.download(name), err_msg=name)
    finally:
        for g in a + b:
            g.close()


def test_batch_rejects_mixed_storage(gpulib):
    from soapbubble_gb300._lib import SoapBubbleError
    from soapbubble_gb300.bubble import GpuBatch
    a, _ = _bubble(16, "c0", 1, 0)
    b, _ = _bubble(16, "c0", 2, 1)
    try:
        with pytest.raises(SoapBubbleError, match="storage"):
            GpuBatch([a, b])
    finally:
        a.close()
        b.close()
