"""GPU checks of the serving loop: requests that arrive while others run
are admitted into the running set, every request completes, and each
result is the same as running that request alone (bit for bit, since a
bubble stepped inside a set matches the same bubble stepped alone)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _requests(n, **kw):
    from soapbubble_gb300 import serve
    return serve.make_requests(n, rate=kw.pop("rate", 400.0), seed=kw.pop("seed", 3),
                               sizes=(16, 32), big=64, big_frac=0.3, steps_range=(12, 37), **kw)


@pytest.mark.parametrize("budget_members", [0, 1], ids=["roomy", "one_at_a_time"])
def test_results_same_alone_and_in_the_mix(gpulib, budget_members):
    from soapbubble_gb300 import serve
    reqs = _requests(7)
    pay = {r.rid: serve.payload(r) for r in reqs}
    # a budget below every request: each is admitted only when nothing else
    # is resident
    budget = 1.0 if budget_members else 150e9
    srv = serve.Server(budget, keep_eta=True)
    res = srv.run(reqs, pay)
    assert [r.rid for r in res] == [r.rid for r in reqs]
    if budget_members:
        assert srv.max_members == 1
    else:
        assert srv.max_members >= 2  # requests overlapped on the GPU
    for q, r in zip(reqs, res):
        assert r.completed >= r.admitted >= 0 and r.latency > 0
        alone = serve.run_alone(q, pay[q.rid])
        np.testing.assert_array_equal(r.eta, alone.eta, err_msg=f"request {q.rid}")
        assert np.isfinite(r.eta).all()
    s = serve.summarise(reqs, res, srv)
    assert s["requests"] == 7 and s["value"] > 0 and s["latency_p99_s"] >= s["latency_p50_s"]
