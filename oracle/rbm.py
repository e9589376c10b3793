"""Oracle: RBM log-amplitude, local energy and Jacobian (test infrastructure only).

* ``log_cosh`` restates ``netket/nn/activation.py:78-84``.
* ``logpsi`` restates ``RBM.__call__`` (``netket/models/rbm.py:57-81``):
  ``sum_j log_cosh(b_j + sum_i s_i W_ij) + a . s``.
* ``local_energies`` restates ``local_value_kernel_jax``
  (``netket/vqs/mc/kernels.py:62-71``): full log-amplitude on every padded
  connected state, ``sum_k mel_k exp(logpsi(x'_k) - logpsi(x))``.
* ``jacobian`` is the analytic per-sample derivative of the RBM in NetKet's
  ravel order ``[Dense.bias (M), Dense.kernel (N*M row-major), visible_bias (N)]``
  (``netket/jax/_jacobian/logic.py:48-384`` with ``mode="real"``), optionally
  centred by the sample mean (``logic.py:364-384``).

Parameters are a dict ``{"bias": (M,), "kernel": (N, M), "visible_bias": (N,)}``.
"""
import numpy as np


def log_cosh(x):
    x = np.abs(x)
    return x + np.log1p(np.exp(-2.0 * x)) - np.log(2.0)


def init_params(rng, N, alpha=1, std=0.01, dtype=np.float64):
    """Normal(0, std) init of all three leaves (``rbm.py:29, 50-55``)."""
    M = int(alpha * N)
    return {
        "bias": rng.normal(0, std, size=M).astype(dtype),
        "kernel": rng.normal(0, std, size=(N, M)).astype(dtype),
        "visible_bias": rng.normal(0, std, size=N).astype(dtype),
    }


def ravel(params):
    return np.concatenate([params["bias"].ravel(), params["kernel"].ravel(),
                           params["visible_bias"].ravel()])


def unravel(flat, N, M):
    flat = np.asarray(flat)
    return {"bias": flat[:M].copy(), "kernel": flat[M:M + N * M].reshape(N, M).copy(),
            "visible_bias": flat[M + N * M:].copy()}


def theta(params, x):
    return np.asarray(x, dtype=np.float64) @ params["kernel"] + params["bias"]


def logpsi(params, x):
    x = np.asarray(x, dtype=np.float64)
    return log_cosh(theta(params, x)).sum(axis=-1) + x @ params["visible_bias"]


def local_energies(params, x, get_conn):
    xp, mels = get_conn(x)
    lp = logpsi(params, x)
    lpp = logpsi(params, xp.reshape(-1, xp.shape[-1])).reshape(mels.shape)
    return np.sum(mels * np.exp(lpp - lp[:, None]), axis=-1)


def jacobian(params, x, center=False):
    """Dense (n, P) real Jacobian d logpsi / d theta."""
    x = np.asarray(x, dtype=np.float64)
    t = np.tanh(theta(params, x))
    n, N = x.shape
    M = t.shape[1]
    O = np.concatenate([t, (x[:, :, None] * t[:, None, :]).reshape(n, N * M), x], axis=1)
    if center:
        O = O - O.mean(axis=0, keepdims=True)
    return O


def forces_and_grad(params, x, eloc):
    """``forces_expect_hermitian`` (``netket/vqs/mc/mc_state/expect_forces.py:68-111``)
    and ``force_to_grad`` (``netket/vqs/mc/common.py:103-118``) for real params:
    grad = 2 Re[(1/n) O^T (E - mean E)]."""
    O = jacobian(params, x)
    de = eloc - eloc.mean()
    F = O.T @ de / len(eloc)
    return F, 2.0 * F
