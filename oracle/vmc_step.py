"""Oracle: one VMC_SR step of the reference algorithm, vectorised with numpy
(test / CPU-baseline infrastructure only).

Same algorithm as the loop-based oracle modules, written for speed so that it
is a fair CPU baseline of the reference:
  * sampling: full RBM forward of every chain for every proposal
    (``netket/sampler/metropolis.py:416-464``), Exchange rule with the
    hoppable-cluster correction (``netket/sampler/rules/exchange.py:143-184``);
  * local energies: padded connected states of 2-site spin-1/2 terms (the
    ``LocalOperatorJax`` order, ``netket/operator/_local_operator/jax.py:74-201``)
    and the full log-amplitude of every row (``netket/vqs/mc/kernels.py:62-71``);
  * statistics (``netket/stats/mc_stats_old.py``);
  * dense centred Jacobian, ``T = O_L O_L^T + lambda I``, Cholesky solve and
    ``delta = O_L^T aux`` (``netket/_src/ngd/srt.py:22-96``);
  * SGD.
``timed_step`` returns the wall time of each phase; ``measured_full_step``
times the full-size step without modelling how any phase grows with size.
"""
import time

import numpy as np
import scipy.linalg as sla

from . import rbm as orbm
from . import stats as ost


def two_site_tables(op):
    """(acting_on (T,2), diag (T,4), offdiag mel (T,4), target row (T,4)) for an
    oracle LocalOperator whose terms all act on 2 sites with <= 1 off-diagonal
    entry per row."""
    P = op.pack()
    assert len(P["groups"]) == 1 and P["groups"][0]["acting_on"].shape[1] == 2
    g = P["groups"][0]
    assert g["ncmax"] <= 1
    T = g["acting_on"].shape[0]
    mel = np.zeros((T, 4))
    tgt = np.zeros((T, 4, 2), dtype=np.int8)
    for t in range(T):
        for r in range(4):
            if g["n_conns"][t, r] > 0:
                mel[t, r] = g["mels"][t, r, 0]
                tgt[t, r] = 1 - 2 * g["x_prime"][t, r, 0]
    return g["acting_on"], g["diag_mels"], mel, tgt, P["max_conn_size"], op.constant


def conn_two_site(x, tables, cutoff=1e-10):
    """Vectorised padded get_conn for 2-site terms (equal to the loop version)."""
    aon, diag, mel, tgt, K, const = tables
    n, N = x.shape
    ids = (x[:, aon] < 0).astype(np.int64)            # (n, T, 2)
    row = 2 * ids[:, :, 0] + ids[:, :, 1]              # (n, T)
    T = aon.shape[0]
    tidx = np.arange(T)[None, :]
    d = const + diag[tidx, row].sum(axis=1)
    m = mel[tidx, row]                                 # (n, T)
    cand_m = np.concatenate([d[:, None], m], axis=1)   # (n, 1+T)
    keep = np.abs(cand_m) > cutoff
    order = np.argsort(~keep, axis=1, kind="stable")[:, :K]
    kept = np.take_along_axis(keep, order, axis=1)
    mels = np.where(kept, np.take_along_axis(cand_m, order, axis=1), 0.0)
    xp = np.repeat(x[:, None, :], K, axis=1)
    term = order - 1                                   # -1 = diagonal
    b, k = np.nonzero(kept & (term >= 0))
    t = term[b, k]
    r = row[b, t]
    xp[b, k, aon[t, 0]] = tgt[t, r, 0]
    xp[b, k, aon[t, 1]] = tgt[t, r, 1]
    return xp, mels


def sample_exchange(params, x, rng, clusters, n_discard, chain_length, sweep):
    B, N = x.shape
    lp = 2 * orbm.logpsi(params, x)
    out = np.empty((B, chain_length, N), dtype=np.int8)
    rows = np.arange(B)
    for step in range(n_discard + chain_length):
        for _ in range(sweep):
            mask = x[:, clusters[:, 0]] != x[:, clusters[:, 1]]
            cnt = mask.sum(1)
            r = np.floor(rng.random(B) * np.maximum(cnt, 1))
            pick = np.argmax(np.cumsum(mask, axis=1) > r[:, None], axis=1)
            u, v = clusters[pick, 0], clusters[pick, 1]
            xp = x.copy()
            xp[rows, u], xp[rows, v] = x[rows, v], x[rows, u]
            cnt2 = (xp[:, clusters[:, 0]] != xp[:, clusters[:, 1]]).sum(1)
            with np.errstate(divide="ignore", invalid="ignore"):
                corr = np.log(cnt) - np.log(cnt2)
            lpp = 2 * orbm.logpsi(params, xp)
            with np.errstate(over="ignore", invalid="ignore"):
                acc = (rng.random(B) < np.exp(lpp - lp + corr)) & (cnt > 0)
            x = np.where(acc[:, None], xp, x)
            lp = np.where(acc, lpp, lp)
        if step >= n_discard:
            out[:, step - n_discard] = x
    return out, x


def timed_step(params, x_chains, rng, clusters, tables, n_discard, chain_length, diag_shift, lr):
    """One minSR step; returns (new params, new chains, energy Stats, phase times)."""
    N = x_chains.shape[1]
    M = params["bias"].shape[0]
    t = {}
    t0 = time.perf_counter()
    samples, x_chains = sample_exchange(params, x_chains, rng, clusters, n_discard, chain_length, N)
    t1 = time.perf_counter()
    x = samples.reshape(-1, N)
    xp, mels = conn_two_site(x, tables)
    lp = orbm.logpsi(params, x)
    lpc = orbm.logpsi(params, xp.reshape(-1, N)).reshape(mels.shape)
    e = np.sum(mels * np.exp(lpc - lp[:, None]), axis=1)
    st = ost.statistics(e.reshape(x_chains.shape[0], -1))
    t2 = time.perf_counter()
    n = x.shape[0]
    O = orbm.jacobian(params, x, center=True) / np.sqrt(n)
    t3 = time.perf_counter()
    T = O @ O.T
    T[np.diag_indices(n)] += diag_shift
    t4 = time.perf_counter()
    dv = 2 * (e - e.mean()) / np.sqrt(n)
    c, low = sla.cho_factor(T, lower=False, overwrite_a=True, check_finite=False)
    aux = sla.cho_solve((c, low), dv, check_finite=False)
    t5 = time.perf_counter()
    delta = O.T @ aux
    flat = orbm.ravel(params) - lr * delta
    t6 = time.perf_counter()
    t = {"sample": t1 - t0, "eloc": t2 - t1, "jacobian": t3 - t2, "gram": t4 - t3,
         "solve": t5 - t4, "update": t6 - t5}
    return orbm.unravel(flat, N, M), x_chains, st, t


def full_size_cholesky_seconds(n, diag_shift, rng, rank=256):
    """Wall time of ``cho_factor`` + ``cho_solve`` (``netket/optimizer/solver/
    solvers.py:266-268``) on an n x n FP64 SPD matrix of the minSR form
    G G^T / rank + diag_shift I (synthetic values: the factorisation's cost does
    not depend on them)."""
    G = rng.normal(size=(n, rank))
    T = G @ G.T / rank
    del G
    T[np.diag_indices(n)] += diag_shift
    b = rng.normal(size=n)
    t0 = time.perf_counter()
    c, low = sla.cho_factor(T, lower=False, overwrite_a=True, check_finite=False)
    sla.cho_solve((c, low), b, check_finite=False)
    return time.perf_counter() - t0


def measured_full_step(params, x_chains, rng, clusters, tables, n_discard, chain_length,
                       diag_shift, lr, n_full, chol_seconds):
    """The reference step at n_full samples, every phase measured at the full
    size or as an exact fraction of it:
      * sampling, local energies, Jacobian rows and delta = O_L^T aux act on each
        sample independently: they run on the given slice of chains
        (n_slice = chains x chain_length samples) and the full step is
        n_full / n_slice such slices;
      * T = O_L O_L^T: the slice's rows of T against a full-size O_L (n_full x P,
        the slice's rows repeated), 1 / (n_full / n_slice) of the full product;
      * the n_full x n_full Cholesky: ``chol_seconds`` from
        ``full_size_cholesky_seconds`` (timed once per run).
    Returns (phase seconds of the full step, slice count)."""
    N = x_chains.shape[1]
    M = params["bias"].shape[0]
    t0 = time.perf_counter()
    samples, x_chains = sample_exchange(params, x_chains, rng, clusters, n_discard, chain_length, N)
    t1 = time.perf_counter()
    x = samples.reshape(-1, N)
    xp, mels = conn_two_site(x, tables)
    lp = orbm.logpsi(params, x)
    lpc = orbm.logpsi(params, xp.reshape(-1, N)).reshape(mels.shape)
    e = np.sum(mels * np.exp(lpc - lp[:, None]), axis=1)
    ost.statistics(e.reshape(x_chains.shape[0], -1))
    t2 = time.perf_counter()
    n = x.shape[0]
    reps = n_full // n
    O = orbm.jacobian(params, x, center=True) / np.sqrt(n_full)
    t3 = time.perf_counter()
    O_full = np.tile(O, (reps, 1))
    t4 = time.perf_counter()
    T_rows = O @ O_full.T
    T_rows[np.arange(n), np.arange(n)] += diag_shift
    t5 = time.perf_counter()
    del O_full, T_rows
    aux = rng.normal(size=n)
    t6 = time.perf_counter()
    delta = O.T @ aux
    orbm.ravel(params) - lr * delta
    t7 = time.perf_counter()
    phases = {"sample": reps * (t1 - t0), "eloc": reps * (t2 - t1), "jacobian": reps * (t3 - t2),
              "gram": reps * (t5 - t4), "solve": chol_seconds, "update": reps * (t7 - t6)}
    return phases, reps
