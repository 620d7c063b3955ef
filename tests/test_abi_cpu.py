"""CPU checks of the C ABI library: it loads, exports every symbol that
include/soapbubble.h declares, and its host-only parts work without a GPU."""
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "soapbubble.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(sb_[a-z_0-9]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(gpulib):
    L = gpulib.lib()
    names = declared_symbols()
    assert len(names) >= 15
    for n in names:
        assert hasattr(L, n), n
    assert sorted(gpulib.EXPORTS) == names


def test_default_params_are_config_txt(gpulib):
    from soapbubble_gb300.bubble import default_params
    p = default_params()
    assert (p.radius, p.H, p.nTheta, p.dt, p.DT, p.frames, p.blendCoeff) == \
        (0.05, 1e-6, 256, 0.005, 0.02, 500, 0.5)


def test_bytes_required_scales_with_cells(gpulib):
    from soapbubble_gb300.bubble import bytes_required, make_params
    a = bytes_required(make_params(64, 0.005))
    b = bytes_required(make_params(128, 0.005))
    assert a > 64 * 128 * 4 * 40
    assert 3.5 < b / a < 4.5
    assert bytes_required(make_params(100, 0.005)) == 0  # not a power of two


def test_exr_writer_roundtrip(gpulib, tmp_path):
    import ctypes as C
    from soapbubble_gb300.exr import read_exr
    rng = np.random.Generator(np.random.PCG64(3))
    img = rng.uniform(-3, 70000, size=(8, 16)).astype(np.float32)
    img[0, :4] = [0.0, 1e-6, 6.1e-5, 65504.0]
    path = str(tmp_path / "f.exr")
    rc = gpulib.lib().sb_write_exr_gray(path.encode(), 16, 8,
                                        img.ctypes.data_as(C.POINTER(C.c_float)))
    assert rc == 0
    ch = read_exr(path)
    assert sorted(ch) == ["B", "G", "R"]
    with np.errstate(over="ignore"):  # values above 65504 become inf in half, as in the file
        expect = img.astype(np.float16).astype(np.float32)  # round to nearest even
    for c in "BGR":
        np.testing.assert_array_equal(ch[c], expect)


def test_config_reader(tmp_path):
    from soapbubble_gb300.bubble import read_config
    cfg = tmp_path / "config.txt"
    cfg.write_text("radius 0.05\nH 0.000001\nU 1\ncm 0.5\nGammam 0.000001\nT 298.15\nDs 0.0\n"
                   "rm 0.000000005\nnumberOfGridsInTheta 256\ntimePerStep 0.005\n"
                   "timePerFrame 0.02\nframeNumbers 500\noutputDir ../out/test\n"
                   "thicknessInit null\nAMGconfig ../init/PCGF_F.json\nblendCoeff 0.5\ngpu 0\n")
    c = read_config(str(cfg))
    assert c["nTheta"] == 256 and c["frames"] == 500 and c["thicknessImage"] == ""
    assert c["outputDir"] == "../out/test" and c["blendCoeff"] == 0.5 and c["device"] == 0


@pytest.mark.parametrize("field,value,msg", [
    ("nTheta", 100, "power of two"), ("nTheta", 2048, "power of two"),
    ("radius", -1.0, "positive"), ("dt", 0.0, "timePerStep"),
    ("storage", 5, "storage"), ("solver_precond", 3, "solver_precond")])
def test_invalid_params_are_rejected_before_any_device_work(gpulib, field, value, msg):
    """sb_create validates its parameters first: a bad configuration is an
    SB_ERR_INVALID with a message, on any machine."""
    import ctypes as C
    from soapbubble_gb300._lib import SB_ERR_INVALID
    from soapbubble_gb300.bubble import make_params
    p = make_params(64, 0.005)
    setattr(p, field, value)
    h = C.c_void_p()
    L = gpulib.lib()
    assert L.sb_create(C.byref(p), C.byref(h)) == SB_ERR_INVALID
    assert not h.value
    assert msg in L.sb_last_error().decode()


def test_null_handles_and_members_are_rejected(gpulib):
    """Entry points check their handles before any device work: a null
    bubble, or a batch with a null member or no members, is an
    SB_ERR_INVALID with a message, on any machine."""
    import ctypes as C
    from soapbubble_gb300._lib import SB_ERR_INVALID
    L = gpulib.lib()
    out = C.c_void_p()
    for members in ([None], [None, None]):
        arr = (C.c_void_p * len(members))(*members)
        assert L.sb_batch_create(arr, len(members), C.byref(out)) == SB_ERR_INVALID
        assert not out.value
        assert "valid bubbles" in L.sb_last_error().decode()
    arr = (C.c_void_p * 1)(None)
    assert L.sb_batch_create(arr, 0, C.byref(out)) == SB_ERR_INVALID
    # a member listed twice is refused before any member is read (the
    # handles here are never dereferenced)
    fake = C.c_void_p(0x1000)
    arr = (C.c_void_p * 3)(0x2000, fake, fake)
    assert L.sb_batch_create(arr, 3, C.byref(out)) == SB_ERR_INVALID
    assert not out.value
    assert "twice" in L.sb_last_error().decode()
    assert L.sb_step(None, 1, 0.0, 0.005) == SB_ERR_INVALID
    assert L.sb_run(None, None, 1) == SB_ERR_INVALID
    assert L.sb_wait_staged(None) == SB_ERR_INVALID
    assert L.sb_batch_step(None, 1, 0.0, 0.005) == SB_ERR_INVALID
    buf = (C.c_double * 4)()
    assert L.sb_download_system(None, 0, buf, 4) == SB_ERR_INVALID
    L.sb_default_params(None)  # ignored, no crash
    assert L.sb_bytes_required(None) == 0
