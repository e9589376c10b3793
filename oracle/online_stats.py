"""Oracle: streaming Monte Carlo statistics (test infrastructure only).

Restates NetKet's online accumulator in FP64 numpy:

* ``update`` -- ``netket/_src/stats/online_stats/kernels.py:123-190``: per-chain
  parallel Welford merge (optional exponential decay of the old counts and
  sums), then the online autocovariance sums of ``_acf_core`` (kernels.py:
  23-107): for every lag ``k <= max_lag`` the pairs ``(x_j, x_{j-k})`` inside the
  new batch, plus the pairs whose older member sits in the right-aligned rolling
  buffer of the last ``max_lag`` samples of each chain (at most ``buf_len`` of
  them valid); the buffer is then refilled with the newest samples.
* the read-outs of ``netket/_src/stats/online_stats/accumulator.py:240-447``:
  mean, pooled variance, between-chain tau, ACF (per-lag pair means, averaged
  over chains, normalised by lag 0), Geyer initial-positive / initial-monotone
  tau, split R-hat and the error of the mean.

Real data only (the RBM local estimators are real).  The restatement is pinned
against ``tests/golden/online_stats.npz``, which ``tests/golden/make_golden.py``
produced by executing the reference's own ``_update_arrays`` / ``_acf_core`` and
``OnlineStats`` read-outs on the same inputs.
"""
import math

import numpy as np


def new_state(n_chains, max_lag):
    """Empty accumulator (accumulator.py:93-135)."""
    a = max_lag + 1 if max_lag > 0 else 0
    z = np.zeros
    return dict(count=z(n_chains), mean=z(n_chains), M2=z(n_chains),
                cross=z((n_chains, a)), m1=z((n_chains, a)), m2=z((n_chains, a)),
                pair=z((n_chains, a)), buf=z((n_chains, max_lag)), buf_len=0, n_total=0,
                max_lag=max_lag)


def update(state, data, decay=None):
    """Return a new state with ``data`` (n_chains, n_batch) merged in."""
    s = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in state.items()}
    x = np.asarray(data, dtype=np.float64)
    if x.ndim == 1:
        x = x[None, :]
    C, nb = x.shape
    if C != s["count"].shape[0]:
        raise ValueError(f"Number of chains changed: expected {s['count'].shape[0]}, got {C}")
    L = s["max_lag"]

    # parallel Welford merge (kernels.py:157-172)
    c_mean = x.mean(axis=1)
    c_M2 = ((x - c_mean[:, None]) ** 2).sum(axis=1)
    if decay is not None:
        s["count"] *= decay
        s["M2"] *= decay
    cnt = s["count"]
    new_cnt = cnt + nb
    safe = np.where(new_cnt > 0, new_cnt, 1.0)
    delta = c_mean - s["mean"]
    s["mean"] = s["mean"] + delta * (nb / safe)
    s["M2"] = s["M2"] + c_M2 + delta ** 2 * (cnt * nb / safe)
    s["count"] = new_cnt

    if L > 0:
        if decay is not None:
            for k in ("cross", "m1", "m2", "pair"):
                s[k] *= decay
        old = s["buf_len"]
        buf = state["buf"]
        for k in range(L + 1):
            # pairs inside the batch: j >= k (kernels.py:57-64)
            cur, lag = x[:, k:], x[:, :nb - k] if k < nb else x[:, :0]
            cur = cur[:, :lag.shape[1]]
            w = ((cur * lag).sum(1), lag.sum(1), cur.sum(1), float(max(nb - k, 0)))
            # pairs reaching into the buffer: j < k, j - k >= -old (kernels.py:66-83)
            lo, hi = max(0, k - old), min(k, nb)
            j = np.arange(lo, hi)
            cur_c = x[:, j]
            lag_c = buf[:, L - (k - j)] if len(j) else np.zeros((C, 0))
            c = ((cur_c * lag_c).sum(1), lag_c.sum(1), cur_c.sum(1), float(len(j)))
            s["cross"][:, k] += w[0] + c[0]
            s["m1"][:, k] += w[1] + c[1]
            s["m2"][:, k] += w[2] + c[2]
            s["pair"][:, k] += w[3] + c[3]
        # rolling buffer of the last L samples, right-aligned (kernels.py:96-105)
        if nb >= L:
            s["buf"] = x[:, nb - L:].copy()
        else:
            s["buf"] = np.concatenate([buf[:, nb:], x], axis=1)
    s["buf_len"] = min(s["buf_len"] + nb, L)
    s["n_total"] += C * nb
    return s


# ---------------------------------------------------------------- read-outs
def mean(s):
    tot = s["count"].sum()
    return math.nan if tot == 0 else float((s["count"] * s["mean"]).sum() / tot)


def variance(s):
    tot = s["count"].sum()
    if tot == 0:
        return math.nan
    gm = (s["count"] * s["mean"]).sum() / tot
    return float((s["M2"].sum() + (s["count"] * (s["mean"] - gm) ** 2).sum()) / tot)


def tau_corr_batch(s):
    C = s["count"].shape[0]
    if C < 2:
        return math.nan
    v = variance(s)
    if math.isnan(v) or v <= 0:
        return math.nan
    n_eff = s["n_total"] / C
    return max((n_eff * float(np.var(s["mean"])) / v - 1) * 0.5, 0.0)


def acf(s):
    if s["max_lag"] == 0:
        return None
    n = np.maximum(s["pair"], 1.0)
    cov = (s["cross"] / n - (s["m1"] / n) * (s["m2"] / n)).mean(axis=0)
    if cov[0] <= 0:
        return None
    return cov / cov[0]


def tau_corr_acf(s):
    """Geyer initial positive + initial monotone sequence (accumulator.py:306-330)."""
    rho = acf(s)
    if rho is None:
        return math.nan
    m = len(rho) // 2
    if m == 0:
        return math.nan
    P = rho[0:2 * m:2] + rho[1:2 * m:2]
    bad = np.nonzero(P <= 0)[0]
    if len(bad):
        P = P[:bad[0]]
    if len(P) == 0:
        return 1.0
    P = np.minimum.accumulate(P)
    return max(2.0 * float(P.sum()) - 1.0, 1.0)


def tau_corr(s):
    t = tau_corr_acf(s)
    return tau_corr_batch(s) if math.isnan(t) else t


def R_hat(s):
    C = s["count"].shape[0]
    if C < 2:
        return math.nan
    W = float((s["M2"] / np.maximum(s["count"], 1.0)).mean())
    if W <= 0:
        return math.nan
    N = float(s["count"].mean())
    return math.sqrt((N - 1) / N + float(np.var(s["mean"])) / W)


def error_of_mean(s):
    C = s["count"].shape[0]
    if C > 1:
        return math.sqrt(float(np.var(s["mean"])) / C)
    v = variance(s)
    t = tau_corr_acf(s)
    if not math.isnan(t):
        return math.sqrt(v * t / s["n_total"])
    t = tau_corr_batch(s)
    if not math.isnan(t):
        return math.sqrt(v * (2 * t + 1) / s["n_total"])
    return math.nan


def derived(s):
    """[mean, variance, tau_corr, tau_corr_batch, tau_corr_acf, R_hat, error_of_mean]."""
    return np.array([mean(s), variance(s), tau_corr(s), tau_corr_batch(s), tau_corr_acf(s),
                     R_hat(s), error_of_mean(s)])
