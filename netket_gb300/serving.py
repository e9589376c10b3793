"""Continuous-batching VMC server: ``expect`` / ``expect_and_grad`` requests and
expect-to-tolerance requests over a mix of Hamiltonians, state resident on the
device, admission by HBM budget, p50 / p99 latency.

* A *session* is a variational state (RBM parameters + Metropolis chains) that
  stays on the device between requests; a request names its session and the
  Hamiltonian, and reads the energy statistics (and, for ``expect_and_grad``,
  the gradient ``2 Re[(1/n) O^T (E - mean E)]``) as in
  ``MCState.expect_and_grad`` (``netket/vqs/mc/mc_state/state.py:695-753``).
* Admission: a request enters when a slot (a CUDA stream with its own library
  context) is free and its estimated device footprint fits in what remains of
  the HBM budget; otherwise it waits.  Requests of different sessions run
  concurrently on their slots; requests of one session run in arrival order
  (its chains advance from one request to the next).
* Completion is detected by polling CUDA events, so requests that arrive while
  others are in flight are admitted as soon as a slot and memory free up --
  the device is never drained between requests.
* A request with ``atol`` / ``rtol`` is served as ``MCState.expect_to_precision``
  (``netket/_src/vqs/expect_to_precision.py:70-164``): sampling rounds (the
  first with the discarded sweeps, later ones without) whose local energies
  are merged into an ``OnlineStats`` accumulator on the request's slot, until
  its error of the mean meets the tolerance or ``max_rounds`` is reached.  The
  request keeps its slot between rounds; the accumulator is read only after a
  round's event has completed, so the other slots keep running meanwhile.
* Every request's work is a fixed sequence of deterministic kernels on its own
  data, so its result is the same alone and in any mix.
"""
import heapq
import math
import time
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _native as nat
from . import kernels as K
from .graph import Chain, Square
from .hilbert import Spin
from .models import RBM
from .operator import Heisenberg, Ising
from .sampler import MetropolisExchange, MetropolisLocal
from .online_stats import not_converged, online_statistics
from .stats import Stats
from .vqs import MCState


@dataclass
class ProblemSpec:
    """A Hamiltonian + model family: ``kind`` "tfim" (chain of N, field h) or
    "heisenberg" (L x L square, J1 = 1, Marshall sign rule, Sz = 0)."""
    kind: str
    size: int
    h: float = 1.0
    alpha: int = 1
    n_samples: int = 4096
    seed: int = 0

    @property
    def N(self):
        return self.size if self.kind == "tfim" else self.size * self.size


@dataclass(order=True)
class Request:
    arrival: float
    rid: int
    session: str = field(compare=False)
    spec: ProblemSpec = field(compare=False)
    want_grad: bool = field(compare=False, default=True)
    atol: float = field(compare=False, default=None)
    rtol: float = field(compare=False, default=None)
    max_rounds: int = field(compare=False, default=64)

    @property
    def to_tolerance(self):
        return self.atol is not None or self.rtol is not None


@dataclass
class Result:
    rid: int
    session: str
    stats: Stats
    grad: np.ndarray
    arrival: float
    start: float
    finish: float
    n_samples: int = 0
    rounds: int = 1

    @property
    def latency_ms(self):
        return 1000.0 * (self.finish - self.arrival)


class Session:
    def __init__(self, spec):
        self.spec = spec
        N = spec.N
        if spec.kind == "tfim":
            hi = Spin(0.5, N)
            self.H = Ising(hi, Chain(N), h=spec.h)
            sampler = MetropolisLocal(hi, n_chains=min(1024, spec.n_samples))
        else:
            g = Square(spec.size)
            hi = Spin(0.5, N, total_sz=0)
            self.H = Heisenberg(hi, g, J=1.0, sign_rule=True)
            sampler = MetropolisExchange(hi, graph=g, n_chains=min(1024, spec.n_samples))
        self.vs = MCState(sampler, RBM(alpha=spec.alpha), n_samples=spec.n_samples,
                          n_discard_per_chain=5, seed=spec.seed, sampler_seed=spec.seed + 1,
                          precision="fp32")
        self.busy = False

    def footprint(self):
        """Device bytes one request needs beyond the resident state."""
        vs = self.vs
        n, N, M, P = vs.n_samples, vs.N, vs.M, vs.n_parameters
        chunks = max(1, math.ceil(n / 1024))
        return n * N + n * M * 4 + n * 8 * 4 + P * 8 * (chunks + 2) + (1 << 20)


class _InFlight:
    def __init__(self, req, slot, start, event, host_stats, host_grad, nbytes, acc=None):
        self.req, self.slot, self.start, self.event = req, slot, start, event
        self.host_stats, self.host_grad, self.nbytes = host_stats, host_grad, nbytes
        self.acc, self.rounds = acc, 1


class Server:
    """Continuous-batching executor (see the module docstring)."""

    def __init__(self, hbm_budget_bytes=8 << 30, n_slots=8):
        nat.require_cuda()
        self.budget = int(hbm_budget_bytes)
        self.slots = [torch.cuda.Stream() for _ in range(n_slots)]
        self.free_slots = list(range(n_slots))
        self.sessions = {}
        self.in_use = 0
        self.waiting = []  # heap of requests that arrived
        self.inflight = []
        self.results = []
        self.peak_inflight = 0

    def session(self, name, spec):
        if name not in self.sessions:
            self.sessions[name] = Session(spec)
        return self.sessions[name]

    # ------------------------------------------------------------ one request
    def _round(self, req, slot, acc, first):
        """One sampling round of an expect-to-tolerance request: local energies
        merged into the accumulator on the slot's stream."""
        sess = self.sessions[req.session]
        vs, op = sess.vs, sess.H
        strm = self.slots[slot]
        strm.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(strm), nat.use_ctx(100 + slot):
            if first:
                vs.sample()
            else:
                vs.sample(n_discard_per_chain=0)
            acc = online_statistics(vs.local_estimators(op), acc, max_lag=64)
            ev = torch.cuda.Event()
            ev.record(strm)
        return acc, ev

    def _launch(self, req, slot):
        sess = self.session(req.session, req.spec)
        sess.busy = True
        nbytes = sess.footprint()
        if req.to_tolerance:
            acc, ev = self._round(req, slot, None, True)
            self.in_use += nbytes
            return _InFlight(req, slot, time.perf_counter(), ev, None, None, nbytes, acc)
        vs, op = sess.vs, sess.H
        strm = self.slots[slot]
        strm.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(strm), nat.use_ctx(100 + slot):
            vs.sample()
            x = vs.samples.reshape(-1, vs.N)
            _, _, t = K.rbm_forward(vs.params_c, x, vs.N, vs.M, want_tanh=True)
            e = K.local_energies_fused(op, vs.params_c, x, vs.N, vs.M)
            st = K.stats_device(e.reshape(vs.sampler.n_chains, -1))
            host_stats = torch.empty(5, dtype=torch.float64).pin_memory()
            host_stats.copy_(st, non_blocking=True)
            host_grad = None
            if req.want_grad:
                n = x.shape[0]
                v = K.center_scale(e, st[0:1], 2.0 / n)
                g = K.ot_v(t, x, vs.N, vs.M, v)
                host_grad = torch.empty(g.numel(), dtype=torch.float64).pin_memory()
                host_grad.copy_(g, non_blocking=True)
            ev = torch.cuda.Event()
            ev.record(strm)
        self.in_use += nbytes
        return _InFlight(req, slot, time.perf_counter(), ev, host_stats, host_grad, nbytes)

    def _admit(self):
        deferred = []
        while self.waiting and self.free_slots:
            req = heapq.heappop(self.waiting)
            sess = self.sessions.get(req.session)
            if sess is not None and sess.busy:
                deferred.append(req)  # one request per session at a time, in arrival order
                continue
            if sess is None:
                sess = self.session(req.session, req.spec)
            if self.inflight and self.in_use + sess.footprint() > self.budget:
                deferred.append(req)  # the oldest waiting request does not fit yet
                break
            slot = self.free_slots.pop()
            self.inflight.append(self._launch(req, slot))
            self.peak_inflight = max(self.peak_inflight, len(self.inflight))
        for r in deferred:
            heapq.heappush(self.waiting, r)

    def _retire(self):
        done = [f for f in self.inflight if f.event.query()]
        finished = 0
        for f in done:
            req = f.req
            if req.to_tolerance:
                with torch.cuda.stream(self.slots[f.slot]):
                    st = f.acc.get_stats()  # the round's event has completed: no wait
                if not_converged(st, req.atol, req.rtol) and f.rounds < req.max_rounds:
                    f.acc, f.event = self._round(req, f.slot, f.acc, False)
                    f.rounds += 1
                    continue
            self.inflight.remove(f)
            now = time.perf_counter()
            self.free_slots.append(f.slot)
            self.in_use -= f.nbytes
            self.sessions[req.session].busy = False
            finished += 1
            if req.to_tolerance:
                self.results.append(Result(req.rid, req.session, st, None, req.arrival, f.start,
                                           now, f.acc.n_samples, f.rounds))
                continue
            grad = f.host_grad.numpy().copy() if f.host_grad is not None else None
            self.results.append(Result(req.rid, req.session,
                                       Stats.from_array(f.host_stats.numpy()), grad,
                                       req.arrival, f.start, now, req.spec.n_samples))
        return finished

    def serve(self, requests, t0=None):
        """Run a request stream whose ``arrival`` times are seconds after t0."""
        pending = sorted(requests)
        t0 = time.perf_counter() if t0 is None else t0
        for r in pending:
            r.arrival = t0 + r.arrival
        i = 0
        while i < len(pending) or self.waiting or self.inflight:
            now = time.perf_counter()
            while i < len(pending) and pending[i].arrival <= now:
                heapq.heappush(self.waiting, pending[i])
                i += 1
            self._retire()
            self._admit()
            if not self.inflight and not self.waiting and i < len(pending):
                time.sleep(max(0.0, min(0.002, pending[i].arrival - time.perf_counter())))
        torch.cuda.synchronize()
        return sorted(self.results, key=lambda r: r.rid)


def mixed_specs(n, seed=0):
    """Seeded mix: 1D TFIM (N 16-256) and 2D Heisenberg (6x6 .. 16x16), alpha in
    {1, 2, 4}, 2048-16384 samples."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n):
        alpha = int(rng.choice([1, 2, 4]))
        ns = int(rng.choice([2048, 4096, 8192, 16384]))
        if rng.random() < 0.5:
            N = int(rng.choice(np.arange(16, 257, 16)))
            out.append(ProblemSpec("tfim", N, h=float(rng.uniform(0.5, 1.5)), alpha=alpha,
                                   n_samples=ns, seed=int(rng.integers(1 << 30))))
        else:
            L = int(rng.choice(np.arange(6, 17, 2)))
            out.append(ProblemSpec("heisenberg", L, alpha=alpha, n_samples=ns,
                                   seed=int(rng.integers(1 << 30))))
    return out


def poisson_stream(specs, rate_hz, seed=0, sessions=None):
    """Requests with exponential inter-arrival times (rate_hz) over ``specs``;
    request k uses session ``sessions[k]`` (default: one session per spec)."""
    rng = np.random.default_rng(seed)
    t = 0.0
    reqs = []
    for k, spec in enumerate(specs):
        t += rng.exponential(1.0 / rate_hz)
        sname = sessions[k] if sessions is not None else f"s{k}"
        reqs.append(Request(t, k, sname, spec, want_grad=True))
    return reqs


def latency_summary(results, wall_s):
    lat = np.array([r.latency_ms for r in results])
    return {"requests": len(results), "p50_ms": round(float(np.percentile(lat, 50)), 3),
            "p99_ms": round(float(np.percentile(lat, 99)), 3),
            "mean_ms": round(float(lat.mean()), 3),
            "throughput_rps": round(len(results) / wall_s, 3),
            "samples_per_s": round(sum(r.n_samples for r in results) / wall_s, 1)}
