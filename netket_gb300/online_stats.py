"""Streaming Monte Carlo statistics (``netket.stats.OnlineStats``).

``OnlineStats`` mirrors ``netket/_src/stats/online_stats/accumulator.py:30-447``:
per-chain Welford state plus the online autocovariance sums of the last
``max_lag`` lags, merged batch by batch.  The merge runs on the GPU
(``vmck_online_stats_update``, one warp per chain); the read-outs (mean,
variance, ACF, Geyer tau, R-hat, error of the mean) are small reductions over
the (n_chains,) and (n_chains, max_lag + 1) state and run as torch operations
on the device the state lives on.

As in the reference the accumulator is a value: ``update`` returns a new
``OnlineStats`` and leaves the old one untouched.  ``online_statistics``,
``expand_max_lag`` and ``thin_acf_by_2`` follow
``netket/_src/stats/online_stats/operations.py``; ``OnlineStatsBatch`` and the
delta method follow ``accumulator_batch.py``.  Real data only: the local
estimators of the real RBM are real (complex input raises ``TypeError``).
"""
import math

import numpy as np
import torch

from . import _native as nat
from . import kernels as K
from .stats import Stats

_KEYS = ("count", "mean", "M2", "cross", "m1", "m2", "pair", "buf")


def _as_device_2d(data):
    if isinstance(data, LocalEstimators):
        data = data.data
    if isinstance(data, torch.Tensor):
        t = data
    else:
        a = np.asarray(data)
        if np.iscomplexobj(a):
            raise TypeError("OnlineStats: complex data is not supported on this path")
        t = torch.as_tensor(a)
    if t.is_complex():
        raise TypeError("OnlineStats: complex data is not supported on this path")
    if t.ndim == 1:
        t = t[None, :]
    if t.ndim != 2:
        raise ValueError(f"data must be 1D or 2D, got {t.ndim}D")
    return t


class OnlineStats:
    """Streaming accumulator of MCMC statistics over successive batches.

    ``OnlineStats(n_chains, dtype, decay=None, max_lag=64)`` starts empty;
    ``OnlineStats.from_data(batch)`` or ``online_statistics(batch)`` start from
    a first batch of shape ``(n_samples,)`` or ``(n_chains, n_per_chain)``.
    """

    def __init__(self, n_chains, dtype=torch.float64, *, decay=None, max_lag=64, device=None):
        max_lag = int(max_lag)
        if max_lag < 0:
            raise ValueError("max_lag must be >= 0")
        a = max_lag + 1 if max_lag > 0 else 0
        dev = nat.device() if device is None else device
        z = lambda *s: torch.zeros(s, dtype=torch.float64, device=dev)
        self.max_lag = max_lag
        self._decay = decay
        self._dtype = _torch_dtype(dtype)
        self._s = {"count": z(n_chains), "mean": z(n_chains), "M2": z(n_chains),
                   "cross": z(n_chains, a), "m1": z(n_chains, a), "m2": z(n_chains, a),
                   "pair": z(n_chains, a), "buf": z(n_chains, max_lag)}
        self._n_samples_total = 0
        self._buf_len = 0

    # ---------------------------------------------------------------- construction
    @classmethod
    def from_data(cls, data, *, decay=None, max_lag=64):
        t = _as_device_2d(data)
        est = cls(t.shape[0], dtype=t.dtype, decay=decay, max_lag=max_lag)
        return est.update(t)

    def state_dict(self):
        """Host copy of the accumulator (the arrays of ``vmck_online_stats`` plus
        the counters), for checkpoints."""
        d = {k: v.cpu().numpy() for k, v in self._s.items()}
        d.update(max_lag=np.int64(self.max_lag), n_total=np.int64(self._n_samples_total),
                 buf_len=np.int64(self._buf_len),
                 decay=np.float64(-1.0 if self._decay is None else self._decay),
                 f32=np.int64(self._dtype == torch.float32))
        return d

    @classmethod
    def from_state_dict(cls, d, device=None):
        """Inverse of ``state_dict`` (onto ``device``, default the CUDA device)."""
        max_lag = int(d["max_lag"])
        decay = float(d["decay"])
        est = object.__new__(cls)
        est.max_lag = max_lag
        est._decay = None if decay < 0 else decay
        est._dtype = torch.float32 if int(d.get("f32", 0)) else torch.float64
        dev = nat.device() if device is None else device
        est._s = {k: torch.as_tensor(np.asarray(d[k], dtype=np.float64), device=dev).contiguous()
                  for k in _KEYS}
        C = est._s["count"].shape[0]
        a = max_lag + 1 if max_lag > 0 else 0
        for k in ("cross", "m1", "m2", "pair"):
            est._s[k] = est._s[k].reshape(C, a)
        est._s["buf"] = est._s["buf"].reshape(C, max_lag)
        est._n_samples_total = int(d["n_total"])
        est._buf_len = int(d["buf_len"])
        return est

    def _replace(self, **kw):
        new = object.__new__(OnlineStats)
        new.__dict__.update(self.__dict__)
        new._s = dict(self._s)
        for k, v in kw.items():
            setattr(new, k, v)
        return new

    def update(self, data):
        """Merge a batch ``(n_samples,)`` or ``(n_chains, n_per_chain)`` and
        return the updated accumulator (accumulator.py:160-223)."""
        t = _as_device_2d(data)
        C, nb = t.shape
        if C != self.n_chains:
            raise ValueError(f"Number of chains changed: expected {self.n_chains}, got {C}")
        if nb == 0:
            raise ValueError("update needs at least one sample per chain")
        dev = self._s["count"].device
        s = {k: v.clone() for k, v in self._s.items()}
        decay = 1.0 if self._decay is None else float(self._decay)
        K.online_stats_update(t.to(device=dev, dtype=torch.float64), s, self.max_lag,
                              self._buf_len, decay, self._dtype == torch.float32)
        new = self._replace(_n_samples_total=self._n_samples_total + C * nb,
                            _buf_len=min(self._buf_len + nb, self.max_lag))
        new._s = s
        return new

    # ---------------------------------------------------------------- state views
    @property
    def n_chains(self):
        return self._s["count"].shape[0]

    @property
    def decay(self):
        return 1.0 if self._decay is None else self._decay

    @property
    def n_samples(self):
        """Total number of samples merged (never decayed)."""
        return self._n_samples_total

    @property
    def chain_means(self):
        return self._chain_mean

    @property
    def _chain_mean(self):
        return self._s["mean"].to(self._dtype)

    @property
    def _chain_count(self):
        return self._s["count"]

    @property
    def _chain_M2(self):
        return self._s["M2"]

    @property
    def _cross_sum(self):
        return self._s["cross"]

    @property
    def _m1_sum(self):
        return self._s["m1"]

    @property
    def _m2_sum(self):
        return self._s["m2"]

    @property
    def _pair_count(self):
        return self._s["pair"]

    @property
    def _chain_buf(self):
        return self._s["buf"]

    # ---------------------------------------------------------------- read-outs
    @property
    def mean(self):
        c, m = self._s["count"], self._s["mean"]
        tot = float(c.sum())
        if tot == 0.0:
            return math.nan
        return float((c * m).sum() / tot)

    @property
    def variance(self):
        c, m = self._s["count"], self._s["mean"]
        tot = float(c.sum())
        if tot == 0.0:
            return math.nan
        gm = (c * m).sum() / tot
        return float((self._s["M2"].sum() + (c * (m - gm) ** 2).sum()) / tot)

    @property
    def tau_corr(self):
        """ACF-based tau when available, else the between-chain estimate."""
        t = self.tau_corr_acf
        return self.tau_corr_batch if math.isnan(t) else t

    @property
    def tau_corr_batch(self):
        """tau = (n B / W - 1) / 2 from the variance of the chain means
        (accumulator.py:270-304)."""
        if self.n_chains < 2:
            return math.nan
        v = self.variance
        if math.isnan(v) or v <= 0:
            return math.nan
        n_eff = self._n_samples_total / self.n_chains
        B = float(self._s["mean"].var(unbiased=False))
        return max((n_eff * B / v - 1) * 0.5, 0.0)

    @property
    def acf(self):
        """Normalised autocorrelation (max_lag + 1,), averaged over chains, from
        the per-lag pair means (accumulator.py:332-355); None without data."""
        if self.max_lag == 0:
            return None
        n = torch.clamp(self._s["pair"], min=1.0)
        cov = (self._s["cross"] / n - (self._s["m1"] / n) * (self._s["m2"] / n)).mean(dim=0)
        c0 = float(cov[0])
        if c0 <= 0:
            return None
        return cov / c0

    @property
    def tau_corr_acf(self):
        """Geyer initial positive + initial monotone sequence estimate
        (accumulator.py:306-330)."""
        rho = self.acf
        if rho is None:
            return math.nan
        r = rho.cpu().numpy()
        m = len(r) // 2
        if m == 0:
            return math.nan
        P = r[0:2 * m:2] + r[1:2 * m:2]
        bad = np.nonzero(P <= 0)[0]
        if len(bad):
            P = P[:bad[0]]
        if len(P) == 0:
            return 1.0
        P = np.minimum.accumulate(P)
        return max(2.0 * float(P.sum()) - 1.0, 1.0)

    @property
    def R_hat(self):
        if self.n_chains < 2:
            return math.nan
        W = float((self._s["M2"] / torch.clamp(self._s["count"], min=1.0)).mean())
        if W <= 0:
            return math.nan
        N = float(self._s["count"].mean())
        B = float(self._s["mean"].var(unbiased=False))
        return math.sqrt((N - 1) / N + B / W)

    def _error_of_mean(self, variance):
        if self.n_chains > 1:
            return math.sqrt(float(self._s["mean"].var(unbiased=False)) / self.n_chains)
        t = self.tau_corr_acf
        if not math.isnan(t):
            return math.sqrt(variance * t / self._n_samples_total)
        t = self.tau_corr_batch
        if not math.isnan(t):
            return math.sqrt(variance * (2 * t + 1) / self._n_samples_total)
        return math.nan

    def get_stats(self):
        if float(self._s["count"].sum()) == 0.0:
            return Stats()
        v = self.variance
        return Stats(mean=self.mean, error_of_mean=self._error_of_mean(v), variance=v,
                     tau_corr=self.tau_corr, R_hat=self.R_hat)

    def to_dict(self):
        return self.get_stats().to_dict()

    def to_compound(self):
        return self.get_stats().to_compound()

    def __repr__(self):
        return repr(self.get_stats())


def _torch_dtype(dt):
    if isinstance(dt, torch.dtype):
        return dt
    return {np.dtype(np.float32): torch.float32, np.dtype(np.float64): torch.float64}.get(
        np.dtype(dt), torch.float64)


def not_converged(stats, atol, rtol):
    """True while ``stats.error_of_mean`` exceeds ``atol`` (absolute) or ``rtol``
    (relative to |mean|; a zero mean gives 0 or inf), as ``_check_not_converged``
    and ``_rel_err`` (``netket/_src/vqs/expect_to_precision.py:26-41``): the
    comparisons are ``>``, so a NaN error stops the sampling."""
    err, scale = abs(stats.error_of_mean), abs(stats.mean)
    if atol is not None and err > atol:
        return True
    if rtol is not None:
        rel = (0.0 if err == 0.0 else math.inf) if scale == 0.0 else err / scale
        if rel > rtol:
            return True
    return False


def online_statistics(data, old_estimator=None, *, decay=None, max_lag=64):
    """Merge ``data`` into ``old_estimator`` (a new accumulator when None)
    (operations.py:51-126).  A ``LocalEstimatorsBatch`` goes to
    ``online_statistics_batch``."""
    if isinstance(data, LocalEstimatorsBatch):
        if old_estimator is not None and not isinstance(old_estimator, OnlineStatsBatch):
            raise TypeError("Mismatch between batched data and non-batched accumulator.")
        return online_statistics_batch(data.data, data.combinator, old_estimator,
                                       max_lag=max_lag)
    if isinstance(old_estimator, OnlineStatsBatch):
        raise TypeError("Mismatch between non-batched data and batched accumulator.")
    t = _as_device_2d(data)
    if old_estimator is None:
        old_estimator = OnlineStats(t.shape[0], dtype=t.dtype, decay=decay, max_lag=max_lag)
    return old_estimator.update(t)


def expand_max_lag(estimator, new_max_lag):
    """Widen the ACF window to ``new_max_lag`` (operations.py:129-190): old lags
    are kept exactly, new lags start with no pairs, the buffer is left-padded so
    its valid samples stay right-aligned."""
    old, new_max_lag = estimator.max_lag, int(new_max_lag)
    if new_max_lag <= old:
        raise ValueError(f"new_max_lag={new_max_lag} must be > current max_lag={old}")
    extra = new_max_lag + 1 - (old + 1 if old > 0 else 0)
    s = dict(estimator._s)
    for k in ("cross", "m1", "m2", "pair"):
        s[k] = torch.nn.functional.pad(s[k], (0, extra))
    s["buf"] = torch.nn.functional.pad(s["buf"], (new_max_lag - old, 0))
    new = estimator._replace(max_lag=new_max_lag)
    new._s = s
    return new


def thin_acf_by_2(estimator):
    """Keep the even lags as the lags of a 2x coarser sweep (operations.py:
    193-261); the buffer keeps every other sample."""
    old = estimator.max_lag
    if old < 2:
        raise ValueError(f"max_lag={old} must be >= 2 to thin by 2")
    new_lag = old // 2
    cols = torch.arange(new_lag + 1, device=estimator._s["count"].device) * 2
    s = dict(estimator._s)
    for k in ("cross", "m1", "m2", "pair"):
        s[k] = s[k][:, cols].contiguous()
    s["buf"] = s["buf"][:, old - 2 * new_lag::2].contiguous()
    new = estimator._replace(max_lag=new_lag, _buf_len=estimator._buf_len // 2)
    new._s = s
    return new


# -------------------------------------------------------------------- K channels
class StatsBatch:
    """Mean and error of an array-valued functional (``netket.stats.StatsBatch``)."""

    def __init__(self, mean, error_of_mean):
        self.mean = mean
        self.error_of_mean = error_of_mean

    def __repr__(self):
        return f"StatsBatch(mean={self.mean}, error_of_mean={self.error_of_mean})"


def _delta_method_stats(f, X, Cov):
    """Var[f_i(X)] ~ J_i^T Cov J_i with J = df/dX (accumulator_batch.py:31-68;
    the reference differentiates forward, here reverse: the same Jacobian)."""
    X = torch.as_tensor(X, dtype=torch.float64)
    mean = f(X)
    scalar = torch.as_tensor(mean).ndim == 0
    if Cov is None:
        if scalar:
            return Stats(mean=float(mean), error_of_mean=math.nan)
        return StatsBatch(mean, torch.full_like(torch.as_tensor(mean), math.nan))
    J = torch.autograd.functional.jacobian(f, X)  # (*out_shape, K)
    var = torch.einsum("...k,kl,...l->...", J, Cov, J)
    err = torch.sqrt(torch.clamp(var, min=0.0))
    if scalar:
        return Stats(mean=float(mean), error_of_mean=float(err))
    return StatsBatch(mean, err)


class OnlineStatsBatch:
    """K per-channel accumulators and a combinator ``f: (K,) -> scalar | array``
    whose error comes from the delta method (accumulator_batch.py:71-228)."""

    def __init__(self, estimators, combinator):
        self.estimators = tuple(estimators)
        self.combinator = combinator

    @classmethod
    def from_data(cls, data, combinator, *, max_lag=64):
        t = data if isinstance(data, torch.Tensor) else torch.as_tensor(np.asarray(data))
        if t.ndim != 3:
            raise ValueError(f"data must be 3D, got {t.ndim}D")
        ests = tuple(OnlineStats(t.shape[0], dtype=torch.float64, max_lag=max_lag)
                     for _ in range(t.shape[-1]))
        return cls(ests, combinator).update(t)

    def update(self, data):
        t = data if isinstance(data, torch.Tensor) else torch.as_tensor(np.asarray(data))
        return OnlineStatsBatch(tuple(e.update(t[..., k]) for k, e in
                                      enumerate(self.estimators)), self.combinator)

    @property
    def n_samples(self):
        return self.estimators[0].n_samples

    @property
    def n_chains(self):
        return self.estimators[0].n_chains

    def _X(self):
        return torch.tensor([e.mean for e in self.estimators], dtype=torch.float64)

    @property
    def mean(self):
        return self.combinator(self._X())

    @property
    def error_of_mean(self):
        return self.get_stats().error_of_mean

    def get_stats(self):
        X = self._X()
        if self.n_chains < 2 or bool(torch.isnan(X).any()):
            return _delta_method_stats(self.combinator, X, None)
        cm = torch.stack([e._s["mean"].to("cpu") for e in self.estimators])
        dev = cm - X[:, None]
        Cov = (dev @ dev.T) / self.n_chains ** 2
        return _delta_method_stats(self.combinator, X, Cov)

    def to_dict(self):
        return self.get_stats().to_dict()

    def to_compound(self):
        return self.get_stats().to_compound()

    def __repr__(self):
        return repr(self.get_stats())


def online_statistics_batch(data, combinator, old_estimator=None, *, max_lag=64):
    if old_estimator is None:
        return OnlineStatsBatch.from_data(data, combinator, max_lag=max_lag)
    return old_estimator.update(data)


# -------------------------------------------------------------------- wrappers
class LocalEstimators:
    """Per-sample local estimators ``(n_chains, chain_len)``
    (``netket/_src/stats/local_estimators.py``)."""

    def __init__(self, data):
        self.data = data

    def to_stats(self):
        from .stats import statistics
        return statistics(self.data)

    def accumulate(self, old=None, *, max_lag=64):
        return online_statistics(self.data, old, max_lag=max_lag)


class LocalEstimatorsBatch:
    """K-channel local estimators ``(n_chains, chain_len, K)`` and their
    combinator."""

    def __init__(self, data, combinator):
        self.data = data
        self.combinator = combinator

    def accumulate(self, old=None, *, max_lag=64):
        return online_statistics_batch(self.data, self.combinator, old, max_lag=max_lag)
