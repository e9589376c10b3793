"""Batched VMC: many independent transverse-field Ising chains of uneven size
stepped together (the "64 instances, N in {16, 24, ..., 144}" workload).

Every instance is exactly the single-problem VMC_SR step of
``netket_gb300.driver`` (RBM, MetropolisLocal, fused local energies, minSR with
the refined FP64 solve) with its own seeds; the batching changes where the work
runs, not what it computes, so an instance's parameters after k steps are
bit-identical to running it alone:

* sampling: one persistent ``vmck_batched_metropolis_local`` launch whose CTAs
  pull (instance, chain group) items, largest N*M first, from an atomic queue;
* local energies: one persistent ``vmck_batched_eloc_ising`` launch, same scheme;
* forward pass, statistics, minSR and SGD: the per-instance kernels;
* the whole step is captured once into a CUDA graph and replayed
  (``capture()`` / ``run()``), so a step costs one graph launch plus one small
  device-to-host read of all energies and solver statuses.

The persistent launch shapes (sampler: chains per work item and CTAs; local
energies: samples per work item and CTAs) are picked by a small autotuner that
times the candidates on the first step and caches the choice per size
signature in ``VMCK_AUTOTUNE_CACHE`` (a JSON file).
"""
import json
import os

import numpy as np
import torch

from . import _native as nat
from . import kernels as K
from .graph import Chain
from .hilbert import Spin
from .models import RBM
from .ngd import minsr_update
from .stats import Stats


def tfim_instances(n_instances=64, sizes=range(16, 145, 8), h_range=(0.5, 1.5), seed=0):
    """(N, h) per instance: N uniform over ``sizes``, h uniform in ``h_range``."""
    rng = np.random.default_rng(seed)
    Ns = rng.choice(np.asarray(list(sizes)), size=n_instances)
    hs = rng.uniform(h_range[0], h_range[1], size=n_instances)
    return [(int(N), float(h)) for N, h in zip(Ns, hs)]


def _device_table(structs):
    raw = bytes(b"".join(bytes(s) for s in structs))
    host = torch.frombuffer(bytearray(raw), dtype=torch.uint8)
    return host.to(nat.device())


def _autotune_cache_path():
    return os.environ.get("VMCK_AUTOTUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "vmck_autotune.json"))


_LAUNCH_KEYS = ("chains_per_item", "sampler_ctas", "samples_per_item", "eloc_ctas")


def _load_tune_cache(path):
    """The autotune cache as a dict; a missing or unreadable file is empty."""
    try:
        with open(path) as f:
            cache = json.load(f)
    except (OSError, ValueError):
        return {}
    return cache if isinstance(cache, dict) else {}


def _cached_launch(cache, sig):
    """The cached launch shape for ``sig`` if it names every launch parameter
    as a positive int, else None (the signature is tuned again)."""
    c = cache.get(sig)
    if not isinstance(c, dict):
        return None
    if not all(isinstance(c.get(k), int) and c[k] > 0 for k in _LAUNCH_KEYS):
        return None
    return c


def _store_tune_choice(path, sig, choice):
    """Add ``sig -> choice`` to the cache file, re-reading it first so entries
    other processes wrote meanwhile are kept, and replacing it atomically."""
    try:
        os.makedirs(os.path.dirname(path) or ".", exist_ok=True)
        cache = _load_tune_cache(path)
        cache[sig] = choice
        tmp = f"{path}.{os.getpid()}.tmp"
        with open(tmp, "w") as f:
            json.dump(cache, f, indent=1)
        os.replace(tmp, path)
    except OSError:
        pass


def _work_lists(Ns, Ms, n_chains, n_samples, chains_per_item, samples_per_item):
    """Flat int32 (instance, first chain) and (instance, first sample) pairs:
    every instance's chains cut into blocks of ``chains_per_item`` and its
    samples into blocks of ``samples_per_item``, largest instances (N * M)
    first so the persistent CTAs end together."""
    order = sorted(range(len(Ns)), key=lambda i: -Ns[i] * Ms[i])
    cw = [(i, b) for i in order for b in range(0, n_chains, chains_per_item)]
    ew = [(i, s) for i in order for s in range(0, n_samples, samples_per_item)]
    return (np.asarray(cw, dtype=np.int32).reshape(-1),
            np.asarray(ew, dtype=np.int32).reshape(-1))


class BatchedTFIM:
    def __init__(self, instances, *, alpha=2, n_chains=1024, chain_length=4, n_discard=5,
                 diag_shift=1e-4, lr=0.01, seed=0, gram_mode=1, refine_iters=4,
                 launch=None, n_streams=8):
        nat.require_cuda()
        self.instances = list(instances)
        self.n_inst = len(self.instances)
        self.alpha, self.B, self.L, self.n_discard = alpha, n_chains, chain_length, n_discard
        self.diag_shift, self.lr, self.gram_mode = diag_shift, lr, gram_mode
        self.refine_iters = refine_iters
        dev = nat.device()
        model = RBM(alpha=alpha, param_dtype=torch.float32)
        self.model = model
        self.N = [N for N, _ in self.instances]
        self.M = [model.n_hidden(N) for N in self.N]
        self.P = [model.n_parameters(N) for N in self.N]
        off = np.concatenate([[0], np.cumsum(self.P)])
        self.p_off = off
        self.p64 = torch.cat([model.init_flat(seed + i, N) for i, N in enumerate(self.N)])
        self.p32 = self.p64.to(torch.float32)
        self.sigma, self.logp, self.nacc, self.samples, self.edges = [], [], [], [], []
        self.eloc = []
        for i, (N, h) in enumerate(self.instances):
            hi = Spin(0.5, N)
            self.sigma.append(hi.random_state(seed + i + 1, self.B, stream_id=1))
            self.logp.append(torch.zeros(self.B, dtype=torch.float64, device=dev))
            self.nacc.append(torch.zeros(self.B, dtype=torch.int64, device=dev))
            self.samples.append(torch.empty((self.B, self.L, N), dtype=torch.int8, device=dev))
            e = np.asarray(Chain(N).edges(), dtype=np.int32)
            self.edges.append(torch.as_tensor(e, device=dev))
            self.eloc.append(torch.empty(self.B * self.L, dtype=torch.float64, device=dev))
        self.seeds = [(seed + i + 1) & (2**64 - 1) for i in range(self.n_inst)]
        self.max_N, self.max_M = max(self.N), max(self.M)
        self.queue = torch.zeros(2, dtype=torch.int32, device=dev)
        self.stats = torch.zeros((self.n_inst, 5), dtype=torch.float64, device=dev)
        self.status = torch.zeros(self.n_inst, dtype=torch.int32, device=dev)
        self._build_tables()
        self.launch = launch or self._autotune()
        self._build_work()
        self.streams = [torch.cuda.Stream() for _ in range(max(1, n_streams))]
        self.graph = None
        self.step_count = 0

    # ------------------------------------------------------------ tables
    def _pslice(self, i, dt):
        src = self.p32 if dt == torch.float32 else self.p64
        return src[self.p_off[i]:self.p_off[i + 1]]

    def _build_tables(self):
        chains, ising = [], []
        for i, (N, h) in enumerate(self.instances):
            chains.append(nat.BatchChainsStruct(
                params=self._pslice(i, torch.float32).data_ptr(),
                sigma=self.sigma[i].data_ptr(), log_prob=self.logp[i].data_ptr(),
                n_accepted=self.nacc[i].data_ptr(), samples=self.samples[i].data_ptr(),
                seed=self.seeds[i], counter=0, N=N, M=self.M[i], n_chains=self.B, sweep_size=N))
            ising.append(nat.BatchIsingStruct(
                params=self._pslice(i, torch.float32).data_ptr(),
                x=self.samples[i].data_ptr(), eloc=self.eloc[i].data_ptr(),
                edges=self.edges[i].data_ptr(), n=self.B * self.L, h=h, J=1.0, N=N, M=self.M[i],
                n_edges=len(self.edges[i]), pad=0))
        self.chain_table = _device_table(chains)
        self.ising_table = _device_table(ising)

    def _build_work(self):
        cw, ew = _work_lists(self.N, self.M, self.B, self.B * self.L,
                             self.launch["chains_per_item"], self.launch["samples_per_item"])
        self.chain_work = torch.as_tensor(cw, device=nat.device())
        self.eloc_work = torch.as_tensor(ew, device=nat.device())

    # ------------------------------------------------------------ kernels
    def _sample(self):
        L = nat.lib()
        nat.check(L.vmck_batched_metropolis_local(
            nat.stream(), nat.F32, nat.ptr(self.chain_table), self.n_inst, nat.ptr(self.chain_work),
            self.chain_work.numel() // 2, self.launch["chains_per_item"], nat.ptr(self.queue),
            self.n_discard, self.L, self.max_N, self.max_M, self.launch["sampler_ctas"]))

    def _local_energies(self):
        L = nat.lib()
        nat.check(L.vmck_batched_eloc_ising(
            nat.stream(), nat.F32, nat.ptr(self.ising_table), self.n_inst, nat.ptr(self.eloc_work),
            self.eloc_work.numel() // 2, self.launch["samples_per_item"],
            nat.ptr(self.queue[1:]), self.max_N, self.max_M, self.launch["eloc_ctas"]))

    def step_kernels(self):
        """One batched VMC_SR step on the current stream (no host synchronisation)."""
        self._sample()
        ts = []
        for i in range(self.n_inst):
            x = self.samples[i].reshape(-1, self.N[i])
            _, _, t = K.rbm_forward(self._pslice(i, torch.float32), x, self.N[i], self.M[i],
                                    want_tanh=True)
            ts.append(t)
        self._local_energies()
        # per-instance statistics, minSR and SGD: instances are independent, so
        # they run concurrently on n_streams streams (fork / join on events),
        # each stream with its own cuBLAS / cuSOLVER context
        main = torch.cuda.current_stream()
        forked = torch.cuda.Event()
        forked.record(main)
        for k, strm in enumerate(self.streams):
            strm.wait_event(forked)
        for i in range(self.n_inst):
            k = i % len(self.streams)
            with torch.cuda.stream(self.streams[k]), nat.use_ctx(k + 1):
                self._instance_update(i, ts[i])
        for strm in self.streams:
            done = torch.cuda.Event()
            done.record(strm)
            main.wait_event(done)

    def _instance_update(self, i, t):
        N, M = self.N[i], self.M[i]
        x = self.samples[i].reshape(-1, N)
        st = K.stats_device(self.eloc[i].reshape(self.B, self.L))
        self.stats[i].copy_(st)
        dp, info = minsr_update(t, x, N, M, self.eloc[i], st[0:1], self.diag_shift,
                                gram_mode=self.gram_mode, solve="refined",
                                refine_iters=self.refine_iters, check=False)
        self.status[i:i + 1].copy_(info["status_dev"])
        K.sgd_(self._pslice(i, torch.float64), dp, self.lr, self._pslice(i, torch.float32))

    # ------------------------------------------------------------ driving
    def capture(self):
        """Run one step eagerly (sizes every workspace), then capture one step."""
        self.step_kernels()
        self.step_count += 1
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            with torch.cuda.graph(g, stream=side):
                self.step_kernels()
        torch.cuda.current_stream().wait_stream(side)
        self.graph = g
        return g

    def step(self):
        """One step (graph replay when captured); returns (energies, statuses)."""
        if self.graph is not None:
            self.graph.replay()
        else:
            self.step_kernels()
        self.step_count += 1
        host = torch.cat([self.stats.reshape(-1), self.status.to(torch.float64)]).cpu().numpy()
        stats = host[:5 * self.n_inst].reshape(self.n_inst, 5)
        status = host[5 * self.n_inst:].astype(np.int64)
        return [Stats.from_array(r) for r in stats], status

    def energies(self):
        return self.stats[:, 0].cpu().numpy()

    def instance_parameters(self, i):
        return self._pslice(i, torch.float64)

    # ------------------------------------------------------------ autotuning
    def _signature(self):
        return f"tfim:{sorted(self.N)}:a{self.alpha}:B{self.B}:L{self.L}"

    def _autotune(self):
        sig = self._signature()
        path = _autotune_cache_path()
        cached = _cached_launch(_load_tune_cache(path), sig)
        if cached is not None:
            return cached
        sms = torch.cuda.get_device_properties(nat.device()).multi_processor_count
        best = None
        # save the chain state: tuning runs advance the chains, restore afterwards
        saved = [s.clone() for s in self.sigma]
        saved_acc = [a.clone() for a in self.nacc]
        for cpi in (2, 4, 8):
            for per_sm in (4, 8, 16):
                cand = {"chains_per_item": cpi, "sampler_ctas": sms * per_sm,
                        "samples_per_item": 8, "eloc_ctas": sms * 8}
                self.launch = cand
                self._build_work()
                self._sample()
                torch.cuda.synchronize()
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record()
                self._sample()
                b.record()
                torch.cuda.synchronize()
                ms = a.elapsed_time(b)
                if best is None or ms < best[0]:
                    best = (ms, dict(cand))
        # local-energy launch shape (a pure function of the samples just drawn)
        self.launch = dict(best[1])
        best_e = None
        for spi in (4, 8, 16):
            for per_sm in (4, 8, 16):
                self.launch.update(samples_per_item=spi, eloc_ctas=sms * per_sm)
                self._build_work()
                self._local_energies()
                torch.cuda.synchronize()
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record()
                self._local_energies()
                b.record()
                torch.cuda.synchronize()
                ms = a.elapsed_time(b)
                if best_e is None or ms < best_e[0]:
                    best_e = (ms, spi, sms * per_sm)
        best[1].update(samples_per_item=best_e[1], eloc_ctas=best_e[2])
        for s, v in zip(self.sigma, saved):
            s.copy_(v)
        for s, v in zip(self.nacc, saved_acc):
            s.copy_(v)
        # the tuning launches advanced the proposal counters: rebuild the tables
        self._build_tables()
        choice = dict(best[1], tuned_ms=round(best[0], 4), tuned_eloc_ms=round(best_e[0], 4))
        _store_tune_choice(path, sig, choice)
        return choice
