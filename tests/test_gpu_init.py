"""GPU checks of the texture initialisers (Solver::initThicknessfromPic and
initAirflowfromPic, kernel/initializer.cu:50-135) on generated EXR
textures of the reference's layout (HALF B, G, R channels, 1024 x 512 or
smaller): the thickness and wind the bubble holds afterwards follow the
reference's formulas on the resampled texture."""
import numpy as np
import pytest

from _exr import resize_linear, write_exr_bgr

pytestmark = pytest.mark.gpu


def _texture(tmp_path, h, w, seed):
    rng = np.random.default_rng(seed)
    b = rng.uniform(0.2, 0.8, (h, w)).astype(np.float16)
    g = rng.uniform(-1.0, 1.0, (h, w)).astype(np.float16)
    r = rng.uniform(-1.0, 1.0, (h, w)).astype(np.float16)
    p = str(tmp_path / "tex.exr")
    write_exr_bgr(p, b, g, r)
    return p, b, g, r


@pytest.mark.parametrize("storage", [0, 1], ids=["fp32", "bf16"])
def test_thickness_from_texture(gpulib, tmp_path, storage):
    from soapbubble_gb300.bubble import GpuBubble, make_params
    nT = 64
    p, b, _, _ = _texture(tmp_path, 512, 1024, 5)
    with GpuBubble(make_params(nT, 0.005, storage=storage)) as gb:
        gb.init_thickness_from_exr(p)
        c = resize_linear(b.astype(np.float32), 2 * nT, nT).astype(np.float64)
        want = ((c - 0.5) * 0.3 + 0.5).astype(np.float32)
        eta = gb.download("eta").astype(np.float32)
        if storage == 0:
            np.testing.assert_array_equal(eta, want)
        else:
            # BF16 deviations from the (BF16-rounded) mean: within half a BF16
            # spacing of the deviation
            dev = np.abs(want - np.float32(np.mean(want))) + 2.0 ** -8
            assert np.all(np.abs(eta - want) <= 2.0 ** -8 * dev + 1e-6)
        # the BIMOCQ reference fields restart from the new thickness
        np.testing.assert_array_equal(gb.download("eta_init"), gb.download("eta"))
        assert not gb.download("eta_delta").any()
        gb.step(2, 0.0, 0.005)
        assert np.isfinite(gb.download("eta")).all()


def test_airflow_from_texture(gpulib, tmp_path):
    from soapbubble_gb300.bubble import GpuBubble, make_params
    nT, radius = 32, 0.05
    p, _, g, r = _texture(tmp_path, 32, 64, 6)
    with GpuBubble(make_params(nT, 0.005, radius=radius)) as gb:
        gb.init_airflow_from_exr(p)
        G = resize_linear(g.astype(np.float32), 2 * nT, nT).astype(np.float64)
        R = resize_linear(r.astype(np.float32), 2 * nT, nT).astype(np.float64)
        u = (0.5 * (G + np.roll(G, 1, axis=1)) * radius).astype(np.float32)
        v = (-0.5 * (R[:-1] + R[1:]) * radius).astype(np.float32)
        np.testing.assert_array_equal(gb.download("uair_init").astype(np.float32), u)
        np.testing.assert_array_equal(gb.download("vair_init").astype(np.float32), v)
        gb.init_airflow_from_exr("")  # no texture: zero wind
        assert not gb.download("uair_init").any() and not gb.download("vair_init").any()


def test_missing_texture_keeps_defaults(gpulib, tmp_path):
    from soapbubble_gb300._lib import SB_ERR_IO, SoapBubbleError
    from soapbubble_gb300.bubble import GpuBubble, make_params
    with GpuBubble(make_params(16, 0.005)) as gb:
        gb.init_thickness_from_exr("")
        assert np.all(gb.download("eta") == 0.5)
        with pytest.raises(SoapBubbleError) as e:
            gb.init_thickness_from_exr(str(tmp_path / "none.exr"))
        assert e.value.code == SB_ERR_IO
        assert np.all(gb.download("eta") == 0.5)
