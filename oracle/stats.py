"""Oracle: Monte Carlo statistics, blocking estimator (test infrastructure only).

Restates ``netket/stats/mc_stats_old.py:28-196`` (the default path of
``netket/stats/mc_stats.py:259-301``): population mean/variance, variance of
chain means, block variance with ``l_block = max(1, L // 32)``, the
batch/block/NaN choice for the error and tau, and split-R-hat
``sqrt((L-1)/L + var(half-chain means) / var)``.  FP64 throughout.
"""
from dataclasses import dataclass
import math

import numpy as np


@dataclass
class Stats:
    mean: float
    error_of_mean: float
    variance: float
    tau_corr: float
    R_hat: float

    def as_array(self):
        return np.array([self.mean, self.error_of_mean, self.variance, self.tau_corr,
                         self.R_hat])


def statistics(data, batch_size=32, plain_rhat=False):
    data = np.atleast_1d(np.asarray(data, dtype=np.float64))
    if data.ndim == 1:
        data = data.reshape(1, -1)
    B, L = data.shape
    mean = data.mean()
    variance = data.var()
    ts = data.size

    cm = data.mean(axis=1)
    batch_var, n_batches = cm.var(), cm.size

    l_block = max(1, L // batch_size)
    n_blk = int(math.floor(L / float(l_block)))
    blocks = data[:, : n_blk * l_block].reshape(-1, l_block).mean(axis=1)
    if blocks.size > 0:
        block_var, n_blocks = blocks.var(), blocks.size
    else:
        block_var, n_blocks = np.nan, 0

    with np.errstate(divide="ignore", invalid="ignore"):
        tau_batch = ((ts / n_batches) * batch_var / variance - 1) * 0.5
        tau_block = ((ts / n_blocks) * block_var / variance - 1) * 0.5 if n_blocks else np.nan

    batch_good = (tau_batch < 6 * L) and (n_batches >= batch_size)
    block_good = (tau_block < 6 * l_block) and (n_blocks >= batch_size)
    if batch_good:
        err = math.sqrt(batch_var / n_batches)
        tau = max(tau_batch, 0.0)
    elif block_good:
        err = math.sqrt(block_var / n_blocks)
        tau = max(tau_block, 0.0)
    else:
        err, tau = np.nan, np.nan

    if n_batches > 1:
        if not plain_rhat:
            if L % 2 == 0:
                half = data.reshape(2 * B, L // 2)
            else:
                half = data[:, :-1].reshape(2 * B, L // 2)
            batch_var = half.mean(axis=1).var()
        with np.errstate(divide="ignore", invalid="ignore"):
            R_hat = math.sqrt((L - 1) / L + batch_var / variance) if variance > 0 else np.nan
    else:
        R_hat = np.nan
    return Stats(float(mean), float(err), float(variance), float(tau), float(R_hat))
