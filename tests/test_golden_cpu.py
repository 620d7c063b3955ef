"""The oracle reproduces the committed golden step fixtures (CPU only).

The fixtures (tests/golden/*.npz, made by tests/golden/make_golden.py) hold
an FP32-exact input state and the FP64 oracle's output after one step.
"""
import glob
import os

import numpy as np
import pytest

# the oracle-made step fixtures (the reference-made ref_* and the texture
# fixture have their own tests)
GOLDEN = sorted(p for p in glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz"))
                if not os.path.basename(p).startswith(("ref_", "tex_")))


def switches(meta):
    """radius and the plain_advection / single_step_velocity / viscous
    switches of a fixture (fixtures without them: radius 1, all off)."""
    if len(meta) < 11:
        return 1.0, 0, 0, 0
    return float(meta[7]), int(meta[8]), int(meta[9]), int(meta[10])


def load_case(oracle, path):
    z = np.load(path)
    nT, dt, t, strict, force = z["meta"][:5]
    radius, plain, single, viscous = switches(z["meta"])
    nT = int(nT)
    p = oracle.default_params(nT, radius=radius, dt_s=float(dt))
    p.t, p.strict, p.force_reinit, p.nthreads = float(t), int(strict), int(force), 1
    p.plain_advection, p.single_step_velocity, p.viscous = plain, single, viscous
    a = {k[3:]: z[k].astype(np.float64) for k in z.files if k.startswith("in_")}
    ob = oracle.OracleBubble(p, a["eta"], a["gamma"], a["uth"], a["uph"], a["uair_init"],
                             a["vair_init"])
    for k, v in a.items():
        ob.a[k][...] = v
    return z, ob


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(g) for g in GOLDEN])
def test_oracle_reproduces_golden(oracle, path):
    z, ob = load_case(oracle, path)
    st = ob.step()
    assert st.reinit == int(z["meta"][5])
    for k in z.files:
        if not k.startswith("out_"):
            continue
        ref = z[k]
        got = ob.a[k[4:]]
        scale = max(np.max(np.abs(ref)), 1e-30)
        assert np.max(np.abs(got - ref)) / scale < 1e-10, k
