"""Oracle: SR / minSR natural-gradient updates and dense solvers
(test infrastructure only).

* ``prepare_input``: ``netket/_src/ngd/sr_srt_common.py:45-101``
  (``O_L = O_c / sqrt(n)``, ``dv = 2 (E - mean E) / sqrt(n)``, real mode).
* ``srt_update`` (minSR): ``netket/_src/ngd/srt.py:22-96``
  (``T = O_L O_L^T + lambda I [+ proj_reg/n 11^T]``, ``delta = O_L^T T^-1 dv``,
  SPRING momentum).
* ``sr_update``: ``netket/_src/ngd/sr.py:23-80``
  (``(O_L^T O_L + lambda I) delta = O_L^T dv``, momentum).
* ``cholesky``, ``pinv_smooth``, ``cholesky_with_fallback``:
  ``netket/optimizer/solver/solvers.py:33-139, 242-340`` and
  ``netket/_src/solvers/nan_fallback.py:22-45``.
* ``sgd``: ``optax.sgd`` as used by ``netket/optimizer/__init__.py:33-60``:
  ``theta <- theta - lr * delta``.
"""
import numpy as np
import scipy.linalg as sla


def prepare_input(O, eloc):
    n = O.shape[0]
    de = eloc - np.sum(eloc / n)
    dv = 2.0 * de * np.sqrt(1.0 / n)
    return O * np.sqrt(1.0 / n), dv


def cholesky(A, b):
    c, low = sla.cho_factor(A, lower=False)
    return sla.cho_solve((c, low), b), None


def pinv_smooth(A, b, rtol=1e-14, rtol_smooth=1e-14):
    if not np.all(np.isfinite(A)):  # XLA's eigh returns NaN rather than raising
        nan = np.full(A.shape[0], np.nan)
        return nan, {"eval_min": np.nan, "eval_max": np.nan, "rank": 0,
                     "cond_number": np.nan}
    s, U = np.linalg.eigh(A)
    rel = np.abs(s / s[-1])
    with np.errstate(divide="ignore"):
        s_inv = np.where(rel > rtol, 1.0 / s, 0.0)
        reg = 1.0 / (1.0 + (rtol_smooth / rel) ** 6)
    s_inv = s_inv * reg
    x = U @ (s_inv * (U.T @ b))
    info = {"eval_min": s[0], "eval_max": s[-1], "rank": int(np.sum(s > rtol * s[-1])),
            "cond_number": s[-1] / s[0]}
    return x, info


def cholesky_with_fallback(A, b, rtol=1e-14, rtol_smooth=1e-14):
    bad_in = bool(np.any(np.isnan(b)) or np.any(np.isnan(A)))
    try:
        x, _ = cholesky(A, b)
        bad_out = bool(np.any(~np.isfinite(x)))
    except (np.linalg.LinAlgError, ValueError):
        x, bad_out = None, True
    if bad_in or bad_out:
        x, _ = pinv_smooth(A, b, rtol, rtol_smooth)
        return x, {"solver_fallback": True}
    return x, {"solver_fallback": False}


def srt_update(O_c, eloc, diag_shift, solver=cholesky_with_fallback, proj_reg=None,
               momentum=None, old_updates=None):
    """minSR update from the centred Jacobian ``O_c`` (n, P).  With ``momentum``
    (SPRING, ``srt.py:34-35, 79-82``): ``dv -= momentum O_L old`` and the update
    gains ``momentum old``; returns (update, info) or, with momentum,
    (update, info, new old_updates = update)."""
    O_L, dv = prepare_input(O_c, eloc)
    if momentum is not None:
        old = np.zeros(O_L.shape[1]) if old_updates is None else np.asarray(old_updates)
        dv = dv - momentum * (O_L @ old)
    T = O_L @ O_L.T
    T = T + diag_shift * np.eye(T.shape[0])
    if proj_reg is not None:
        T = T + proj_reg / T.shape[0]
    aux, info = solver(T, dv)
    upd = O_L.T @ aux
    if momentum is None:
        return upd, info
    upd = upd + momentum * old
    return upd, info, upd


def sr_update(O_c, eloc, diag_shift, solver=cholesky_with_fallback, momentum=None,
              old_updates=None):
    """SR update; with ``momentum``: ``F += diag_shift momentum old``
    (``sr.py:43-47``) and the new old_updates is the update."""
    O_L, dv = prepare_input(O_c, eloc)
    F = O_L.T @ dv
    if momentum is not None:
        old = np.zeros(O_L.shape[1]) if old_updates is None else np.asarray(old_updates)
        F = F + diag_shift * momentum * old
    S = O_L.T @ O_L + diag_shift * np.eye(O_L.shape[1])
    x, info = solver(S, F)
    if momentum is None:
        return x, info
    return x, info, x


def sgd(flat_params, update, lr):
    return flat_params - lr * update
