"""Monte Carlo statistics (``netket.stats``): ``Stats`` and ``statistics``.

``statistics(data)`` runs the FP64 blocking estimator of
``netket/stats/mc_stats_old.py:88-196`` on the GPU (``vmck_stats_f64``) and
reads back the five numbers.  ``NETKET_USE_PLAIN_RHAT`` is honoured.
"""
import math
import os

import numpy as np
import torch

from . import _native as nat
from .kernels import stats_device


class Stats:
    """mean, error_of_mean, variance, tau_corr, R_hat (``netket/stats/mc_stats.py:85-181``)."""

    def __init__(self, mean=float("nan"), error_of_mean=float("nan"), variance=float("nan"),
                 tau_corr=float("nan"), R_hat=float("nan")):
        self.mean = mean
        self.error_of_mean = error_of_mean
        self.variance = variance
        self.tau_corr = tau_corr
        self.R_hat = R_hat

    @classmethod
    def from_array(cls, a):
        a = np.asarray(a, dtype=np.float64)
        return cls(*[float(v) for v in a[:5]])

    def to_dict(self):
        return {"Mean": self.mean, "Variance": self.variance, "Sigma": self.error_of_mean,
                "R_hat": self.R_hat, "TauCorr": self.tau_corr}

    def to_compound(self):
        return "Mean", self.to_dict()

    def as_array(self):
        return np.array([self.mean, self.error_of_mean, self.variance, self.tau_corr, self.R_hat])

    def __getitem__(self, k):
        return self.to_dict()[k]

    def __repr__(self):
        def fmt(v):
            return "nan" if not math.isfinite(v) else f"{v:.4g}"
        return (f"{self.mean:.6g} ± {fmt(self.error_of_mean)} [σ²={fmt(self.variance)}, "
                f"R̂={self.R_hat:.4f}]")


def _plain_rhat():
    return os.environ.get("NETKET_USE_PLAIN_RHAT", "0").lower() in ("1", "true", "yes")


def statistics(data):
    """Statistics of ``data`` (n_chains, chain_length), or a single series."""
    if not isinstance(data, torch.Tensor):
        data = torch.as_tensor(np.asarray(data, dtype=np.float64))
    d = data.to(device=nat.device(), dtype=torch.float64)
    if d.ndim == 1:
        d = d.reshape(1, -1)
    if d.ndim != 2:
        raise NotImplementedError("Statistics are implemented only for ndim<=2")
    return Stats.from_array(stats_device(d, _plain_rhat()).cpu().numpy())


from .online_stats import (  # noqa: E402  (re-exported as netket.stats does)
    LocalEstimators, LocalEstimatorsBatch, OnlineStats, OnlineStatsBatch, StatsBatch,
    expand_max_lag, online_statistics, online_statistics_batch, thin_acf_by_2)
