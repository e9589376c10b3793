"""Oracle: Metropolis sampling with Local and Exchange rules
(test infrastructure only).

Restates ``MetropolisSampler._sample_next`` / ``_sample_chain``
(``netket/sampler/metropolis.py:416-505``): ``sweep_size`` proposals per kept
sample, ``log_prob = 2 Re logpsi``, accept when ``u < exp(lp' - lp + corr)``,
samples shaped (n_chains, chain_length, N).  Rules:

* Local (``netket/sampler/rules/local.py:40-49``): flip one uniformly chosen site.
* Exchange (``netket/sampler/rules/exchange.py:143-218``): choose uniformly among
  clusters (i, j) with s_i != s_j, swap, ``corr = log #hoppable(s) - log #hoppable(s')``.

* Hamiltonian (``netket/sampler/rules/hamiltonian.py:84-127``, the numba form):
  choose uniformly among the entries of x's flattened operator row (the
  diagonal entry first whenever the operator has a diagonal; with
  ``diag_rule=2`` only where it is above the cutoff, IsingJax's ``n_conn``,
  ``operator/_ising/jax.py:168-175``), ``corr = log n(x) - log n(x')``.

The random stream is numpy's, so parity with the CUDA sampler (and with NetKet,
whose JAX threefry stream cannot run here) is distributional only, as in
NetKet's own tests (``test/sampler/test_sampler.py:400-458``).
"""
import numpy as np

from . import rbm


def _hoppable(x, clusters):
    return x[:, clusters[:, 0]] != x[:, clusters[:, 1]]


def hamiltonian_row(op, x, diag_rule=1):
    """Candidate states of each row of x (list of (k, N) arrays), numba order."""
    P = op.pack()
    rows = []
    for xs, ms in op.get_conn_flattened_numba_order(x):
        if P["nonzero_diagonal"] and (diag_rule == 0 or
                                      (diag_rule == 2 and not abs(ms[0]) > op.mel_cutoff)):
            xs = xs[1:]
        rows.append(xs)
    return rows


def hamiltonian_propose(op, x, u, diag_rule=1):
    """Proposal and log-correction for uniforms u (``_choose``, hamiltonian.py:
    118-127, then ``- log n_conn(x')``)."""
    x = np.asarray(x, dtype=np.int8)
    rows = hamiltonian_row(op, x, diag_rule)
    prop = x.copy()
    corr = np.zeros(len(x))
    for b, xs in enumerate(rows):
        n = len(xs)
        if n == 0:
            corr[b] = np.nan
            continue
        prop[b] = xs[int(np.floor(u[b] * n))]
        corr[b] = np.log(n)
    n_new = np.array([len(r) for r in hamiltonian_row(op, prop, diag_rule)], dtype=np.float64)
    with np.errstate(divide="ignore"):
        return prop, corr - np.log(n_new)


def sample_chain(params, x, rng, chain_length, sweep_size=None, rule="local",
                 clusters=None, n_discard=0, operator=None, diag_rule=1):
    x = np.array(x, dtype=np.int8)
    B, N = x.shape
    sweep_size = N if sweep_size is None else sweep_size
    lp = 2.0 * rbm.logpsi(params, x)
    out = np.empty((B, chain_length, N), dtype=np.int8)
    n_acc = np.zeros(B, dtype=np.int64)
    rows = np.arange(B)
    for step in range(n_discard + chain_length):
        for _ in range(sweep_size):
            xp = x.copy()
            if rule == "local":
                i = rng.integers(0, N, size=B)
                xp[rows, i] = -xp[rows, i]
                corr = 0.0
            elif rule == "hamiltonian":
                xp, corr = hamiltonian_propose(operator, x, rng.random(B), diag_rule)
            else:
                mask = _hoppable(x, clusters)
                cnt = mask.sum(axis=1)
                r = np.floor(rng.random(B) * np.maximum(cnt, 1)).astype(np.int64)
                pick = np.array([np.flatnonzero(mask[b])[r[b]] if cnt[b] > 0 else 0
                                 for b in range(B)])
                u, v = clusters[pick, 0], clusters[pick, 1]
                xu, xv = x[rows, u].copy(), x[rows, v].copy()
                xp[rows, u], xp[rows, v] = xv, xu
                cnt2 = _hoppable(xp, clusters).sum(axis=1)
                with np.errstate(divide="ignore", invalid="ignore"):
                    corr = np.log(cnt.astype(np.float64)) - np.log(cnt2.astype(np.float64))
            lpp = 2.0 * rbm.logpsi(params, xp)
            with np.errstate(over="ignore", invalid="ignore"):
                acc = rng.random(B) < np.exp(lpp - lp + corr)
            x = np.where(acc[:, None], xp, x)
            lp = np.where(acc, lpp, lp)
            n_acc += acc
        if step >= n_discard:
            out[:, step - n_discard] = x
    return out, x, lp, n_acc


def pauli_hamiltonian_propose(operators, weights, x, u, cutoff=1e-10):
    """Hamiltonian rule for PauliStrings (the jax rule, ``hamiltonian.py:
    153-213``, whose draw set equals ``n_conn`` for PauliStrings): uniform over
    the nonzero slots of x's padded row, ``corr = log n(x) - log n(x')``."""
    from .operator import pauli_get_conn_padded
    x = np.asarray(x, dtype=np.int8)
    xp, mels, n = pauli_get_conn_padded(x, operators, weights, cutoff)
    prop = x.copy()
    for b in range(len(x)):
        nz = np.flatnonzero(mels[b])
        if len(nz):
            prop[b] = xp[b, nz[int(np.floor(u[b] * len(nz)))]]
    _, _, n2 = pauli_get_conn_padded(prop, operators, weights, cutoff)
    with np.errstate(divide="ignore"):
        return prop, np.log(n.astype(np.float64)) - np.log(n2.astype(np.float64))
