"""The soapBubble CLI end to end (kernel/main.cu:4-56, Bubble::run
kernel/bubble.cu:2607-2704) on the reference's config.txt.

The test writes the 17 keys of the shipped config.txt (radius 0.05, nTheta
256, dt 0.005 s, DT 0.02 s, thickness init/midFrequency.exr, blend 0.5)
with frameNumbers reduced to 3 and the output directory in a temporary
folder, and lays out ../init/ next to the run directory as the reference's
build directory has it: midFrequency.exr and velocityfield_512.exr hold the
shipped textures already resampled to the grid (tests/golden/
tex_256x512.npz, FLOAT samples; the reader's resampling is then the
identity).  It runs the built binary, checks frame0000..0002.exr, and
compares the last frame (HALF samples of eta H 2e5) with the FP64 oracle
stepped through the same two frames from the same initial fields.
"""
import os
import subprocess

import numpy as np
import pytest

from _exr import write_exr_bgr

pytestmark = pytest.mark.gpu

CONFIG = """radius 0.05
H 0.000001
U 1
cm 0.5
Gammam 0.000001
T 298.15
Ds 0.0
rm 0.000000005
numberOfGridsInTheta 256
timePerStep 0.005
timePerFrame 0.02
frameNumbers 3
outputDir ../out
thicknessInit ../init/midFrequency.exr
AMGconfig ../init/PCGF_F.json
blendCoeff 0.5
gpu 0
"""


def test_cli_runs_config_txt(gpulib, oracle, tmp_path):
    from soapbubble_gb300 import build
    from soapbubble_gb300.exr import read_exr
    golden = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    tex = np.load(os.path.join(golden, "tex_256x512.npz"))
    B, G, R = tex["thickness_B"], tex["airflow_G"], tex["airflow_R"]
    init, run = tmp_path / "init", tmp_path / "run"
    init.mkdir()
    run.mkdir()
    write_exr_bgr(str(init / "midFrequency.exr"), B, B, B, "float")
    write_exr_bgr(str(init / "velocityfield_512.exr"), np.zeros_like(G), G, R, "float")
    (run / "config.txt").write_text(CONFIG)
    proc = subprocess.run([build.CLI, "config.txt"], cwd=str(run), capture_output=True, text=True,
                          timeout=600)
    assert proc.returncode == 0, proc.stderr[-2000:]
    out = tmp_path / "out"
    assert sorted(os.listdir(out)) == [f"frame{i:04d}.exr" for i in range(3)]
    # the oracle from the same initial fields, two frames of four steps
    nT, r, dt = 256, 0.05, 0.005
    eta0 = (B.astype(np.float64) - 0.5) * 0.3 + 0.5
    G64, R64 = G.astype(np.float64), R.astype(np.float64)
    uair = 0.5 * (G64 + np.roll(G64, 1, axis=1)) * r
    vair = -0.5 * (R64[:-1] + R64[1:]) * r
    # the library stores FP32 fields: start the oracle from the same values
    f32 = lambda a: a.astype(np.float32).astype(np.float64)
    p = oracle.default_params(nT, radius=r, dt_s=dt)
    p.solver_tol = 1e-12
    ob = oracle.OracleBubble(p, f32(eta0), np.ones((nT, 2 * nT)), np.zeros((nT - 1, 2 * nT)),
                             np.zeros((nT, 2 * nT)), f32(uair), f32(vair))
    first = read_exr(str(out / "frame0000.exr"))["B"]
    np.testing.assert_allclose(first, (f32(eta0) * 1e-6 * 2e5).astype(np.float16), rtol=1e-3)
    T = 0.0
    for i in range(1, 3):
        tf = T
        while T + dt <= i * 0.02:
            ob.p.t = tf
            ob.step()
            T += dt
        T = i * 0.02
    last = read_exr(str(out / "frame0002.exr"))
    expect = ob.a["eta"] * 1e-6 * 2e5
    for c in "BGR":  # three equal HALF channels
        np.testing.assert_allclose(last[c], expect, rtol=2e-3, atol=1e-4)
