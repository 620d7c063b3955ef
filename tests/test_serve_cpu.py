"""Request stream generation of the serving loop (CPU only)."""
import numpy as np


def test_request_stream_is_seeded_and_in_range():
    from soapbubble_gb300 import serve
    a = serve.make_requests(500, rate=20.0, seed=1)
    b = serve.make_requests(500, rate=20.0, seed=1)
    assert [(r.arrival, r.nTheta, r.steps, r.seed) for r in a] == \
           [(r.arrival, r.nTheta, r.steps, r.seed) for r in b]
    arr = np.array([r.arrival for r in a])
    assert (np.diff(arr) > 0).all()
    # Poisson stream at 20/s: mean gap 0.05 s
    assert abs(np.diff(arr).mean() - 0.05) < 0.01
    sizes = {r.nTheta for r in a}
    assert sizes <= {64, 128, 256, 512, 1024}
    big = sum(r.nTheta == 1024 for r in a) / len(a)
    assert 0.01 < big < 0.1
    assert all(50 <= r.steps <= 500 for r in a)
    assert all(0.5 <= r.gs_scale <= 1.5 and 0.5 <= r.M_scale <= 1.5 for r in a)


def test_admission_respects_the_batch_limits():
    """sb_batch_create rejects more than 1024 members or a row-table weight
    sum nTheta (2 nTheta + 256) of 2^32 or more; the serving loop admits a
    request only while the set stays within both."""
    from soapbubble_gb300 import serve
    from soapbubble_gb300.bubble import BATCH_MAX_WEIGHT, batch_weight
    assert serve.fits_batch([], 1024)
    assert serve.fits_batch([64] * 1023, 64)
    assert not serve.fits_batch([64] * 1024, 64)
    # with grids of at most 1024 rows the member limit binds first
    assert 1024 * batch_weight(1024) < BATCH_MAX_WEIGHT
    assert serve.fits_batch([1024] * 1023, 1024)
    assert not serve.fits_batch([1024] * 1024, 512)
