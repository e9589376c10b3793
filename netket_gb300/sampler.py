"""Metropolis samplers (``netket.sampler``): ``MetropolisSampler`` with the
``LocalRule`` / ``ExchangeRule`` / ``HamiltonianRule`` transition rules and the
``MetropolisLocal`` / ``MetropolisExchange`` / ``MetropolisHamiltonian``
constructors.

The whole chain (discarded plus kept sweeps) runs in ONE launch of
``vmck_metropolis_sample``: a warp per chain, the RBM pre-activations kept
in shared memory and updated per proposal.  Samples come back shaped
(n_chains, chain_length, N) as in ``netket/sampler/metropolis.py:496-500``.
The random stream is Philox4x32-10, keyed by the sampler seed, with a
proposal counter carried in the sampler state.
"""
import ctypes
from dataclasses import dataclass

import numpy as np
import torch

from . import _native as nat


class MetropolisRule:
    code = None

    def device_clusters(self):
        return None, 0


class LocalRule(MetropolisRule):
    """Flip one uniformly chosen site (``netket/sampler/rules/local.py:40-49``)."""
    code = 0

    def __repr__(self):
        return "LocalRule()"


class ExchangeRule(MetropolisRule):
    """Swap the spins of a uniformly chosen cluster (i, j) with x_i != x_j
    (``netket/sampler/rules/exchange.py:143-218``).  Clusters are all pairs
    with graph distance <= d_max, in row-major order."""
    code = 1

    def __init__(self, *, clusters=None, graph=None, d_max=1, probabilities=None):
        if probabilities is not None:
            probabilities = np.atleast_1d(probabilities)
            if not np.all(probabilities > 0):
                raise ValueError("Probabilities must be positive")
            if not np.allclose(probabilities, probabilities.flat[0]):
                raise NotImplementedError(
                    "ExchangeRule: non-uniform cluster probabilities are not supported")
        if (clusters is None) == (graph is None):
            raise ValueError("You must either provide the list of exchange-clusters or a netket "
                             "graph, from which clusters will be computed using the maximum "
                             "distance d_max.")
        if clusters is None:
            dist = np.asarray(graph.distances())
            cl = np.argwhere(dist <= d_max)
            clusters = cl[cl[:, 0] < cl[:, 1]]
        self.clusters = np.asarray(clusters, dtype=np.int64).reshape(-1, 2)
        self._dev = {}

    def device_clusters(self):
        d = torch.cuda.current_device()
        if d not in self._dev:
            self._dev[d] = torch.as_tensor(self.clusters.astype(np.int32), device=nat.device())
        return self._dev[d], len(self.clusters)

    def __repr__(self):
        return f"ExchangeRule(# of clusters: {len(self.clusters)})"


class HamiltonianRule(MetropolisRule):
    """Move to one of the entries of x's operator row, chosen uniformly, with
    the correction log n(x) - log n(x') (``netket/sampler/rules/hamiltonian.py:
    99-235``).  The operator is an ``Ising`` (its diagonal slot counts only where
    the diagonal element is nonzero, as IsingJax's ``n_conn``) or a
    ``LocalOperator`` (the slot counts whenever the operator has a diagonal,
    as LocalOperator's ``n_conn``; the numba rule draws among the same
    entries).  The reference's jax rule draws among the nonzero entries but
    normalises by ``n_conn``: where a LocalOperator's diagonal element is
    exactly zero that selects no entry and proposes an all-zero row; here the
    zero diagonal entry proposes x itself, as the numba rule does.  For
    ``PauliStrings`` n(x) is the number of slots with a nonzero matrix element
    (PauliStringsJax's ``n_conn``)."""
    code = 2

    def __init__(self, operator):
        from .operator import Ising, LocalOperator, PauliStrings
        self._pauli = isinstance(operator, PauliStrings)
        if self._pauli:
            self._local, self.diag_rule = operator, None
        elif isinstance(operator, Ising):
            self._local = operator.to_local_operator()
            self.diag_rule = 2
        elif isinstance(operator, LocalOperator):
            self._local = operator
            self.diag_rule = 1 if operator._pack()["nonzero_diag"] else 0
        else:
            raise TypeError("Argument to HamiltonianRule must be a valid operator, "
                            f"but operator is a {type(operator)}.")
        self.operator = operator
        self.status = None

    def device_op(self):
        return self._local.device_struct()

    def __repr__(self):
        return f"HamiltonianRule(operator={self.operator})"


@dataclass
class MetropolisSamplerState:
    """Chain state (``netket/sampler/metropolis.py:42-95``)."""
    σ: torch.Tensor
    log_prob: torch.Tensor
    seed: int
    counter: int
    n_accepted_proc: torch.Tensor
    n_steps_proc: int = 0

    @property
    def acceptance(self):
        if self.n_steps_proc == 0:
            return None
        return float(self.n_accepted_proc.sum().item()) / self.n_steps_proc

    @property
    def n_accepted(self):
        return int(self.n_accepted_proc.sum().item())

    @property
    def n_steps(self):
        return self.n_steps_proc

    def __repr__(self):
        acc = ""
        if self.n_steps > 0:
            acc = (f"# accepted = {self.n_accepted}/{self.n_steps} "
                   f"({self.acceptance * 100}%), ")
        return f"MetropolisSamplerState({acc}seed = {self.seed}, counter = {self.counter})"


class MetropolisSampler:
    machine_pow = 2
    is_exact = False

    def __init__(self, hilbert, rule, *, n_chains=None, n_chains_per_rank=None, sweep_size=None,
                 reset_chains=False, chunk_size=None, machine_pow=2, dtype=torch.int8):
        """Argument checks of ``netket/sampler/metropolis.py:273-325`` and
        ``sampler/base.py:139-154`` (one device: ``n_chains_per_rank`` is
        ``n_chains``).  ``chunk_size`` is kept and has no effect (the kernels
        stream the chains); only ``machine_pow = 2`` (sampling |psi|^2) is
        implemented."""
        if not isinstance(rule, MetropolisRule):
            raise TypeError(f"The second positional argument, rule, must be a MetropolisRule "
                            f"but `type(rule)={type(rule)}`.")
        if not isinstance(reset_chains, bool):
            raise TypeError("reset_chains must be a boolean.")
        if isinstance(rule, HamiltonianRule) and rule.operator.hilbert != hilbert:
            raise ValueError(f"The hilbert space of the sampler ({hilbert}) and the hilbert "
                             f"space of the operator ({rule.operator.hilbert}) for "
                             "HamiltonianRule must be the same.")
        if isinstance(machine_pow, complex):
            raise ValueError(f"machine_pow ({machine_pow}) must be real")
        if machine_pow < 0:
            raise ValueError(f"machine_pow ({machine_pow}) must be positive")
        if machine_pow != 2:
            raise NotImplementedError("MetropolisSampler: only machine_pow=2 is implemented")
        if n_chains is not None and n_chains_per_rank is not None:
            raise ValueError("Cannot specify both `n_chains` and `n_chains_per_rank`")
        if n_chains is None:
            n_chains = n_chains_per_rank if n_chains_per_rank is not None else 16
        n_chains = max(int(n_chains), 1)
        if chunk_size is not None and n_chains > chunk_size and n_chains % chunk_size != 0:
            raise ValueError(f"Chunk size must divide number of chains per rank, {n_chains}")
        self.hilbert = hilbert
        self.rule = rule
        self.n_chains = n_chains
        self.sweep_size = hilbert.size if sweep_size is None else int(sweep_size)
        self.reset_chains = reset_chains
        self.chunk_size = chunk_size
        self.dtype = dtype

    @property
    def n_batches(self):
        return self.n_chains

    @property
    def n_chains_per_rank(self):
        return self.n_chains

    def init_state(self, machine, params, seed=0):
        σ = self.hilbert.random_state(seed, self.n_chains, stream_id=1)
        lp = torch.full((self.n_chains,), -np.inf, dtype=torch.float64, device=σ.device)
        acc = torch.zeros(self.n_chains, dtype=torch.int64, device=σ.device)
        return MetropolisSamplerState(σ=σ, log_prob=lp, seed=int(seed) & (2**64 - 1), counter=0,
                                      n_accepted_proc=acc)

    def reset(self, machine, params, state=None):
        """Recompute log_prob for the current parameters and zero the counters
        (``netket/sampler/metropolis.py:382-414``); a new state when ``state`` is
        None (``sampler/base.py:289-321``).  With ``reset_chains`` the chains
        first restart from fresh random states, drawn from the Philox stream
        (seed, 2 + proposal counter): a new stream at every reset."""
        if state is None:
            state = self.init_state(machine, params)
        N = self.hilbert.size
        M = machine.sizes_from_flat(params.numel(), N)
        if self.reset_chains:
            state.σ = self.hilbert.random_state(state.seed, self.n_chains,
                                                stream_id=2 + state.counter)
        from .kernels import rbm_forward
        lp, _, _ = rbm_forward(params, state.σ, N, M)
        state.log_prob = 2.0 * lp.to(torch.float64)
        state.n_accepted_proc = torch.zeros_like(state.n_accepted_proc)
        state.n_steps_proc = 0
        return state

    def sample(self, machine, params, *, state=None, chain_length=1, n_discard=0,
               return_log_probabilities=False):
        """Run ``n_discard`` discarded sweeps then ``chain_length`` kept sweeps
        (``sampler/base.py:344-400``: without a state, a new one is initialised
        and reset).  ``params`` is the flat parameter vector in the compute dtype
        (FP64 or FP32).  Returns samples (n_chains, chain_length, N) and the new
        state; with ``return_log_probabilities``, (samples, 2 Re log psi of each
        sample, shape (n_chains, chain_length)) and the state."""
        if state is None:
            state = self.reset(machine, params)
        if return_log_probabilities:
            samples, state = self.sample(machine, params, state=state,
                                         chain_length=chain_length, n_discard=n_discard)
            B, L, N = samples.shape
            lp = machine.apply(params, samples.reshape(-1, N)).to(torch.float64)
            return (samples, 2.0 * lp.reshape(B, L)), state
        N = self.hilbert.size
        M = machine.sizes_from_flat(params.numel(), N)
        B = self.n_chains
        L = int(chain_length)
        samples = torch.empty((B, L, N), dtype=torch.int8, device=state.σ.device)
        if self.rule.code == 2:
            st = self.rule.device_op()
            if self.rule.status is None or self.rule.status.device != state.σ.device:
                self.rule.status = torch.zeros(1, dtype=torch.int32, device=state.σ.device)
            if self.rule._pauli:
                nat.check(nat.lib().vmck_metropolis_hamiltonian_pauli(
                    nat.stream(), nat.dtype_code(params.dtype), nat.ptr(params.contiguous()), N,
                    M, ctypes.byref(st), nat.ptr(state.σ), nat.ptr(state.log_prob),
                    nat.ptr(state.n_accepted_proc), B, self.sweep_size, int(n_discard), L,
                    nat.ptr(samples), state.seed, state.counter, nat.ptr(self.rule.status)))
                state.counter += (int(n_discard) + L) * self.sweep_size
                state.n_steps_proc += (int(n_discard) + L) * self.sweep_size * B
                return samples, state
            nat.check(nat.lib().vmck_metropolis_hamiltonian(
                nat.stream(), nat.dtype_code(params.dtype), nat.ptr(params.contiguous()), N, M,
                ctypes.byref(st), self.rule.diag_rule, nat.ptr(state.σ), nat.ptr(state.log_prob),
                nat.ptr(state.n_accepted_proc), B, self.sweep_size, int(n_discard), L,
                nat.ptr(samples), state.seed, state.counter, nat.ptr(self.rule.status)))
            state.counter += (int(n_discard) + L) * self.sweep_size
            state.n_steps_proc += (int(n_discard) + L) * self.sweep_size * B
            return samples, state
        cl, C = self.rule.device_clusters()
        nat.check(nat.lib().vmck_metropolis_sample(
            nat.stream(), nat.dtype_code(params.dtype), nat.ptr(params.contiguous()), N, M,
            nat.ptr(state.σ), nat.ptr(state.log_prob), nat.ptr(state.n_accepted_proc), B,
            self.sweep_size, int(n_discard), L, nat.ptr(samples), state.seed, state.counter,
            self.rule.code, nat.ptr(cl), C))
        state.counter += (int(n_discard) + L) * self.sweep_size
        state.n_steps_proc += (int(n_discard) + L) * self.sweep_size * B
        return samples, state

    def __repr__(self):
        return (f"MetropolisSampler(rule={self.rule}, n_chains={self.n_chains}, "
                f"sweep_size={self.sweep_size})")


def MetropolisLocal(hilbert, **kwargs):
    return MetropolisSampler(hilbert, LocalRule(), **kwargs)


def MetropolisExchange(hilbert, *, clusters=None, graph=None, d_max=1, probabilities=None,
                       **kwargs):
    return MetropolisSampler(hilbert, ExchangeRule(clusters=clusters, graph=graph, d_max=d_max,
                                                   probabilities=probabilities), **kwargs)


def MetropolisHamiltonian(hilbert, hamiltonian, **kwargs):
    """Moves along the nonzero off-diagonal entries of ``hamiltonian``
    (``netket/sampler/metropolis.py:686-735``); preserves the operator's
    symmetries (Sz for Heisenberg)."""
    return MetropolisSampler(hilbert, HamiltonianRule(hamiltonian), **kwargs)
