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


_ALIASES = {"Mean": "mean", "Variance": "variance", "Sigma": "error_of_mean", "R": "R_hat",
            "TauCorr": "tau_corr", "TauCorrMax": "tau_corr_max"}


def _format_mean_error(value, err, var):
    """"mean ± error [σ²=variance" with the mean shown to the error's first two
    significant digits, in scientific notation for small numbers, as
    ``netket/stats/mc_stats.py:26-74`` prints ``Stats``."""
    if not math.isfinite(abs(value)) or not math.isfinite(err):
        return f"{value:.2e} ± {err:.2e} [σ²={var:.1e}"
    if err == 0.0:
        return f"{value:.3e} [σ²={var:.1e}"
    if abs(value) + abs(err) < 1e-2 or abs(err) <= 1e-7:
        ref = value if value != 0 else err
        e_val = int(math.floor(math.log10(abs(ref))))
        digits = max(e_val - int(math.floor(math.log10(err))), 0) + 1
        scale = 10.0 ** e_val
        return (f"{value / scale:.{digits}f}".rjust(5) + " ± " +
                f"{err / scale:.{digits}f}".rjust(5) + " e" + f"{ref:e}".split("e")[1] +
                f" [σ²={var:.1e}")
    decimals = 15 if err < 1e-15 else max(int(math.ceil(-math.log10(err))), 0) + 1
    return f"{value:.{decimals}f} ± {err:.{decimals}f} [σ²={var:.1e}"


class Stats:
    """mean, error_of_mean, variance, tau_corr, R_hat (``netket/stats/mc_stats.py:85-181``),
    with the reference's alias names (``Mean``, ``Sigma``, ``R``, ...)."""

    tau_corr_max = float("nan")  # only the FFT autocorrelation estimator sets it

    def __init__(self, mean=float("nan"), error_of_mean=float("nan"), variance=float("nan"),
                 tau_corr=float("nan"), R_hat=float("nan")):
        self.mean = mean
        self.error_of_mean = error_of_mean
        self.variance = variance
        self.tau_corr = tau_corr
        self.R_hat = R_hat

    def __getattr__(self, name):
        if name in _ALIASES:
            return getattr(self, _ALIASES[name])
        raise AttributeError(f"'Stats' object has no attribute '{name}'")

    @property
    def shape(self):
        return ()

    def replace(self, **kw):
        d = dict(mean=self.mean, error_of_mean=self.error_of_mean, variance=self.variance,
                 tau_corr=self.tau_corr, R_hat=self.R_hat)
        d.update(kw)
        return Stats(**d)

    def real(self):
        return self.replace(mean=float(np.real(self.mean)))

    def imag(self):
        return self.replace(mean=float(np.imag(self.mean)))

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
        ext = "" if math.isnan(self.R_hat) else f", R̂={self.R_hat:.3f}"
        return _format_mean_error(self.mean, self.error_of_mean, self.variance) + ext + "]"


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
