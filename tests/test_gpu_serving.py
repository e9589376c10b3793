"""Continuous-batching server: every request's energy statistics and gradient
are bit-identical when it is served alone and when it is served in a Poisson
mix where its work overlaps with other requests' on the device; requests of
one session keep their order; the HBM budget bounds the admitted footprint."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def nk():
    import netket_gb300
    netket_gb300._native.require_cuda()
    return netket_gb300


def _specs(nk):
    S = nk.serving.ProblemSpec
    return [S("tfim", 16, h=0.8, alpha=1, n_samples=2048, seed=1),
            S("heisenberg", 6, alpha=2, n_samples=2048, seed=2),
            S("tfim", 48, h=1.2, alpha=2, n_samples=4096, seed=3),
            S("heisenberg", 8, alpha=1, n_samples=2048, seed=4),
            S("tfim", 32, h=1.0, alpha=4, n_samples=2048, seed=5),
            S("heisenberg", 6, alpha=2, n_samples=2048, seed=2),   # same session as #1
            S("tfim", 16, h=0.8, alpha=1, n_samples=2048, seed=1)]  # same session as #0


SESSIONS = ["a", "b", "c", "d", "e", "b", "a"]


def test_results_same_alone_and_in_mix(nk):
    specs = _specs(nk)
    # alone: one request at a time on a fresh server
    alone = {}
    srv = nk.serving.Server(hbm_budget_bytes=4 << 30, n_slots=4)
    for k, (spec, sname) in enumerate(zip(specs, SESSIONS)):
        req = nk.serving.Request(0.0, k, sname, spec, True)
        (res,) = [r for r in srv.serve([req]) if r.rid == k]
        srv.results = []
        alone[k] = res
    # mix: everything arrives within a few milliseconds
    srv2 = nk.serving.Server(hbm_budget_bytes=4 << 30, n_slots=4)
    reqs = nk.serving.poisson_stream(specs, rate_hz=2000.0, seed=0, sessions=SESSIONS)
    mix = {r.rid: r for r in srv2.serve(reqs)}
    assert srv2.peak_inflight > 1, "requests must overlap on the device"
    for k in alone:
        np.testing.assert_array_equal(mix[k].stats.as_array(), alone[k].stats.as_array())
        np.testing.assert_array_equal(mix[k].grad, alone[k].grad)
    # same-session order: the second request sees advanced chains
    assert not np.array_equal(mix[6].grad, mix[0].grad)


def test_budget_limits_concurrency(nk):
    specs = _specs(nk)[:5]
    srv = nk.serving.Server(hbm_budget_bytes=1, n_slots=4)  # admits one at a time
    reqs = nk.serving.poisson_stream(specs, rate_hz=5000.0, seed=1)
    res = srv.serve(reqs)
    assert len(res) == 5 and srv.peak_inflight == 1
    summ = nk.serving.latency_summary(res, 1.0)
    assert summ["p99_ms"] >= summ["p50_ms"] > 0


def test_expect_to_tolerance_request(nk):
    """An rtol request is served as MCState.expect_to_precision: the same rounds
    and the same accumulator as on an identically built state, bit for bit,
    alone and in a mix with gradient requests on other sessions.  (TFIM N = 16
    with near-uniform initial weights: E_loc variance ~16 around ~-16, so
    rtol = 2e-3 takes tens of 1,024-sample rounds.)"""
    S = nk.serving.ProblemSpec
    spec = S("tfim", 16, h=1.0, alpha=1, n_samples=1024, seed=11)
    rtol = 2e-3

    def tol_request(rid, arrival=0.0):
        return nk.serving.Request(arrival, rid, "tol", spec, want_grad=False, rtol=rtol,
                                  max_rounds=500)

    alone = nk.serving.Server(n_slots=4).serve([tol_request(0)])[0]
    sess = nk.serving.Session(spec)
    acc = sess.vs.expect_to_precision(sess.H, rtol=rtol, max_iter=499)
    ref = acc.get_stats()
    assert alone.rounds == sess.vs.last_precision_rounds + 1 >= 2
    np.testing.assert_array_equal(alone.stats.as_array(), ref.as_array())
    assert alone.stats.error_of_mean <= rtol * abs(alone.stats.mean)
    assert alone.n_samples == acc.n_samples

    others = _specs(nk)[:4]
    reqs = nk.serving.poisson_stream(others, rate_hz=2000.0, seed=3,
                                     sessions=["a", "b", "c", "d"])
    reqs.append(tol_request(len(reqs), arrival=reqs[1].arrival))
    srv = nk.serving.Server(hbm_budget_bytes=4 << 30, n_slots=4)
    mix = {r.rid: r for r in srv.serve(reqs)}
    assert srv.peak_inflight > 1
    np.testing.assert_array_equal(mix[len(reqs) - 1].stats.as_array(), alone.stats.as_array())
    assert mix[len(reqs) - 1].rounds == alone.rounds
