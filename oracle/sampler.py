"""Oracle: Metropolis sampling with Local and Exchange rules
(test infrastructure only).

Restates ``MetropolisSampler._sample_next`` / ``_sample_chain``
(``netket/sampler/metropolis.py:416-505``): ``sweep_size`` proposals per kept
sample, ``log_prob = 2 Re logpsi``, accept when ``u < exp(lp' - lp + corr)``,
samples shaped (n_chains, chain_length, N).  Rules:

* Local (``netket/sampler/rules/local.py:40-49``): flip one uniformly chosen site.
* Exchange (``netket/sampler/rules/exchange.py:143-218``): choose uniformly among
  clusters (i, j) with s_i != s_j, swap, ``corr = log #hoppable(s) - log #hoppable(s')``.

The random stream is numpy's, so parity with the CUDA sampler (and with NetKet,
whose JAX threefry stream cannot run here) is distributional only, as in
NetKet's own tests (``test/sampler/test_sampler.py:400-458``).
"""
import numpy as np

from . import rbm


def _hoppable(x, clusters):
    return x[:, clusters[:, 0]] != x[:, clusters[:, 1]]


def sample_chain(params, x, rng, chain_length, sweep_size=None, rule="local",
                 clusters=None, n_discard=0):
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
