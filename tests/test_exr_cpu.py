"""CPU checks of the EXR texture path of the initialisers
(Solver::initThicknessfromPic / initAirflowfromPic): the reader and the
bilinear resampling, through the C ABI's host utility sb_exr_load_resized
(no device work)."""
import numpy as np
import pytest

from _exr import resize_linear, write_exr_bgr


@pytest.fixture(scope="module")
def lib():
    from soapbubble_gb300 import build
    build.build()
    from soapbubble_gb300 import _lib
    return _lib


def _planes(h, w, seed):
    rng = np.random.default_rng(seed)
    return [rng.uniform(-2.0, 3.0, (h, w)).astype(np.float16) for _ in range(3)]


def test_reader_returns_each_half_channel_exactly(lib, tmp_path):
    from soapbubble_gb300.bubble import exr_load_resized
    b, g, r = _planes(32, 64, 1)
    p = str(tmp_path / "t.exr")
    write_exr_bgr(p, b, g, r)
    for name, plane in (("B", b), ("G", g), ("R", r)):
        np.testing.assert_array_equal(exr_load_resized(p, name, 64, 32),
                                      plane.astype(np.float64), err_msg=name)


@pytest.mark.parametrize("src,dst", [((512, 1024), (128, 256)), ((32, 64), (64, 128)),
                                     ((50, 100), (32, 64)), ((64, 128), (64, 128))],
                         ids=["down4", "up2", "fractional", "same"])
def test_resize_matches_half_pixel_bilinear(lib, tmp_path, src, dst):
    from soapbubble_gb300.bubble import exr_load_resized
    b, g, r = _planes(src[0], src[1], 2)
    p = str(tmp_path / "t.exr")
    write_exr_bgr(p, b, g, r)
    got = exr_load_resized(p, "G", dst[1], dst[0])
    want = resize_linear(g.astype(np.float32), dst[1], dst[0]).astype(np.float64)
    np.testing.assert_array_equal(got, want)


def test_downscale_by_two_averages_pixel_pairs(lib, tmp_path):
    from soapbubble_gb300.bubble import exr_load_resized
    b = np.arange(16 * 32, dtype=np.float16).reshape(16, 32) / np.float16(64)
    p = str(tmp_path / "t.exr")
    write_exr_bgr(p, b, b, b)
    got = exr_load_resized(p, "B", 16, 8)
    x = b.astype(np.float64)
    want = 0.25 * (x[0::2, 0::2] + x[0::2, 1::2] + x[1::2, 0::2] + x[1::2, 1::2])
    np.testing.assert_allclose(got, want, rtol=0, atol=1e-6)


def test_unreadable_files_are_io_errors(lib, tmp_path):
    from soapbubble_gb300._lib import SB_ERR_IO, SoapBubbleError
    from soapbubble_gb300.bubble import exr_load_resized
    with pytest.raises(SoapBubbleError) as e:
        exr_load_resized(str(tmp_path / "missing.exr"), "B", 8, 4)
    assert e.value.code == SB_ERR_IO
    p = tmp_path / "zip.exr"
    b, g, r = _planes(4, 8, 3)
    write_exr_bgr(str(p), b, g, r)
    d = bytearray(p.read_bytes())
    k = d.index(b"compression\0compression\0") + len(b"compression\0compression\0") + 4
    d[k] = 3  # ZIP
    p.write_bytes(bytes(d))
    with pytest.raises(SoapBubbleError, match="uncompressed"):
        exr_load_resized(str(p), "B", 8, 4)
    with pytest.raises(SoapBubbleError, match="no channel"):
        write_exr_bgr(str(p), b, g, r)
        exr_load_resized(str(p), "A", 8, 4)
