"""Host-side scheduling of the continuous-batching server, without a GPU.

``Server._admit`` / ``Server._retire`` are driven directly, with the device
work replaced by fakes: a session's footprint is a number, a request's CUDA
event completes after a set number of polls, and an expect-to-tolerance
accumulator's error of the mean shrinks by a set factor per round.  The
invariants checked are the ones the server promises: every request finishes
exactly once; the HBM budget bounds the admitted footprint whenever more than
one request is in flight; at most ``n_slots`` requests are in flight; requests
of one session run one at a time in arrival order; the oldest waiting request
that does not fit blocks the ones behind it; tolerance requests take rounds
until the error meets the tolerance or ``max_rounds``."""
import math

import numpy as np
import pytest
import torch

from netket_gb300 import serving as S
from netket_gb300.stats import Stats


class FakeEvent:
    def __init__(self, polls):
        self.left = int(polls)

    def query(self):
        self.left -= 1
        return self.left < 0


class FakeSession:
    def __init__(self, spec):
        self.spec = spec
        self.busy = False

    def footprint(self):
        return self.spec.n_samples


class FakeAcc:
    def __init__(self, err, shrink, n):
        self.err, self.shrink, self.n_samples = err, shrink, n

    def get_stats(self):
        return Stats(1.0, self.err, 1.0, 0.0, 1.0)


class FakeServer(S.Server):
    def __init__(self, budget, n_slots, polls, shrink=0.5):
        self.budget = budget
        self.slots = [None] * n_slots
        self.free_slots = list(range(n_slots))
        self.sessions = {}
        self.in_use = 0
        self.waiting = []
        self.inflight = []
        self.results = []
        self.peak_inflight = 0
        self.polls = polls  # rid -> polls before the event completes
        self.shrink = shrink
        self.log = []  # (event, rid, session, in_use after, n in flight)

    def session(self, name, spec):
        if name not in self.sessions:
            self.sessions[name] = FakeSession(spec)
        return self.sessions[name]

    def _round(self, req, slot, acc, first):
        if acc is None:
            acc = FakeAcc(1.0, self.shrink, 0)
        else:
            acc.err *= acc.shrink
        acc.n_samples += req.spec.n_samples
        return acc, FakeEvent(self.polls(req.rid))

    def _launch(self, req, slot):
        sess = self.session(req.session, req.spec)
        assert not sess.busy
        sess.busy = True
        nbytes = sess.footprint()
        self.in_use += nbytes
        self.log.append(("start", req.rid, req.session, self.in_use, len(self.inflight) + 1))
        if req.to_tolerance:
            acc, ev = self._round(req, slot, None, True)
            return S._InFlight(req, slot, 0.0, ev, None, None, nbytes, acc)
        st = torch.tensor([float(req.rid), 0.1, 1.0, 0.0, 1.0], dtype=torch.float64)
        return S._InFlight(req, slot, 0.0, FakeEvent(self.polls(req.rid)), st, None, nbytes)

    def run(self, requests, arrivals_per_tick=1):
        """Requests arrive ``arrivals_per_tick`` at a time; each tick retires
        then admits, as ``Server.serve`` does."""
        pending = list(requests)
        ticks = 0
        while pending or self.waiting or self.inflight:
            for _ in range(arrivals_per_tick):
                if pending:
                    S.heapq.heappush(self.waiting, pending.pop(0))
            self._retire()
            self._admit()
            ticks += 1
            assert len(self.inflight) <= len(self.slots)
            if len(self.inflight) > 1:
                assert self.in_use <= self.budget
            assert ticks < 100_000
        return sorted(self.results, key=lambda r: r.rid)


def _spec(n):
    return S.ProblemSpec("tfim", 16, n_samples=int(n))


@pytest.mark.parametrize("seed", range(25))
def test_scheduler_invariants(seed):
    rng = np.random.default_rng(seed)
    n_req = int(rng.integers(1, 40))
    n_sess = int(rng.integers(1, 8))
    budget = int(rng.integers(50, 400))
    sizes = {f"s{k}": int(rng.integers(10, 200)) for k in range(n_sess)}
    reqs = []
    for rid in range(n_req):
        sname = f"s{int(rng.integers(n_sess))}"
        tol = rng.random() < 0.3
        reqs.append(S.Request(float(rid), rid, sname, _spec(sizes[sname]),
                              rtol=(0.1 if tol else None), max_rounds=int(rng.integers(1, 6))))
    polls = {r.rid: int(rng.integers(0, 5)) for r in reqs}
    srv = FakeServer(budget, int(rng.integers(1, 6)), polls.__getitem__)
    res = srv.run(reqs, arrivals_per_tick=int(rng.integers(1, 4)))

    assert [r.rid for r in res] == list(range(n_req))
    assert srv.in_use == 0 and not srv.inflight and not srv.waiting
    assert sorted(srv.free_slots) == list(range(len(srv.slots)))
    for r, q in zip(res, reqs):
        assert r.session == q.session
        if q.to_tolerance:
            # error 1, 0.5, 0.25, 0.125, ...: converged once err <= rtol * |mean| = 0.1
            need = 1 + math.ceil(math.log(1.0 / 0.1, 2))
            assert r.rounds == min(need, q.max_rounds)
            assert r.n_samples == r.rounds * q.spec.n_samples
            assert r.grad is None
        else:
            assert r.rounds == 1 and r.stats.mean == float(q.rid)

    # a session's requests start in arrival order (FakeServer._launch also
    # asserts that the session is idle, so they never overlap)
    starts = [e for e in srv.log if e[0] == "start"]
    for sname in sizes:
        rids = [e[1] for e in starts if e[2] == sname]
        assert rids == sorted(rids)


def test_oldest_request_that_does_not_fit_blocks_the_rest():
    """Budget 100: A (60) runs; B (60) does not fit; C (10) would fit but waits
    behind B, so nothing overtakes the oldest waiting request."""
    polls = {0: 3, 1: 0, 2: 0}
    srv = FakeServer(100, 4, polls.__getitem__)
    reqs = [S.Request(0.0, 0, "A", _spec(60)), S.Request(1.0, 1, "B", _spec(60)),
            S.Request(2.0, 2, "C", _spec(10))]
    srv.run(reqs, arrivals_per_tick=3)
    starts = [e[1] for e in srv.log if e[0] == "start"]
    assert starts == [0, 1, 2]
    # B and C both started only after A retired: A ran alone
    assert srv.log[0][4] == 1 and srv.log[1][4] == 1


def test_busy_session_does_not_block_other_sessions():
    """Two requests of session A then one of B: the second A waits for the first,
    B runs beside the first A."""
    polls = {0: 3, 1: 0, 2: 0}
    srv = FakeServer(10_000, 4, polls.__getitem__)
    reqs = [S.Request(0.0, 0, "A", _spec(10)), S.Request(1.0, 1, "A", _spec(10)),
            S.Request(2.0, 2, "B", _spec(10))]
    srv.run(reqs, arrivals_per_tick=3)
    starts = [(e[1], e[4]) for e in srv.log if e[0] == "start"]
    assert starts[0] == (0, 1) and starts[1] == (2, 2) and starts[2][0] == 1


def test_oversized_request_runs_alone():
    """A request larger than the whole budget is admitted when nothing else is in
    flight (otherwise it would never run)."""
    polls = {0: 1, 1: 1}
    srv = FakeServer(50, 4, polls.__getitem__)
    res = srv.run([S.Request(0.0, 0, "A", _spec(500)), S.Request(1.0, 1, "B", _spec(10))],
                  arrivals_per_tick=2)
    assert [r.rid for r in res] == [0, 1]
    assert [e[4] for e in srv.log if e[0] == "start"] == [1, 1]


def test_stream_helpers_are_seeded():
    a = S.mixed_specs(12, seed=3)
    b = S.mixed_specs(12, seed=3)
    assert a == b
    for s in a:
        assert s.alpha in (1, 2, 4) and s.n_samples in (2048, 4096, 8192, 16384)
        if s.kind == "tfim":
            assert 16 <= s.N <= 256 and 0.5 <= s.h <= 1.5
        else:
            assert 6 <= s.size <= 16 and s.N == s.size ** 2
    r1 = S.poisson_stream(a, 100.0, seed=1)
    r2 = S.poisson_stream(a, 100.0, seed=1)
    assert [r.arrival for r in r1] == [r.arrival for r in r2]
    gaps = np.diff([0.0] + [r.arrival for r in r1])
    assert np.all(gaps > 0) and [r.session for r in r1] == [f"s{k}" for k in range(12)]
    res = [S.Result(k, "s", None, None, 0.0, 0.0, 0.001 * (k + 1), 100) for k in range(100)]
    summ = S.latency_summary(res, 2.0)
    assert summ["requests"] == 100 and summ["throughput_rps"] == 50.0
    assert summ["p50_ms"] == pytest.approx(50.5) and summ["samples_per_s"] == 5000.0
