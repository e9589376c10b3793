"""Optimisers and the SR preconditioner (``netket.optimizer``).

* ``Sgd(learning_rate)``: ``optax.sgd`` as NetKet wraps it
  (``netket/optimizer/__init__.py:33-60``): ``theta <- theta - lr * update``,
  applied by the ``vmck_sgd`` kernel on the FP64 master parameters.
* ``SR(qgt, solver, diag_shift=)``: stochastic reconfiguration
  (``netket/optimizer/sr.py:62-216``) with the QGT chosen as NetKet's
  ``QGTAuto`` chooses it for an RBM (``netket/optimizer/qgt/default.py:58-97``):
  ``QGTOnTheFly`` solved by conjugate gradients unless a dense solver is given,
  else the dense ``S = O_L^T O_L`` (``qgt_jacobian_dense.py``) solved by
  Cholesky with the pinv_smooth fallback.
* ``qgt``: ``QGTAuto``, ``QGTOnTheFly``, ``QGTJacobianDense`` select the form.
* ``solver``: the dense solvers of ``netket/optimizer/solver/solvers.py``
  (``cholesky``, ``cholesky_with_fallback``, ``pinv_smooth``) on device tensors.
"""
import types

import torch

from . import kernels as K
from . import _native as nat
from .ngd import solve_with_fallback, sr_update, sr_update_onthefly


class Sgd:
    def __init__(self, learning_rate):
        self.learning_rate = learning_rate

    def lr(self, step):
        return self.learning_rate(step) if callable(self.learning_rate) else self.learning_rate

    def apply(self, vstate, update_flat, step=0):
        K.sgd_(vstate.flat_parameters, update_flat, self.lr(step))
        vstate.params_changed()

    def __repr__(self):
        return f"Sgd(learning_rate={self.learning_rate})"


def _flat(tree_or_flat, model):
    if isinstance(tree_or_flat, torch.Tensor):
        return tree_or_flat
    return model.flatten(tree_or_flat)


class QGTAuto:
    """Marker: the QGT form NetKet's heuristic picks (``qgt/default.py:58-97``)."""


class QGTOnTheFly:
    """Marker: the matrix-free QGT, S v by a JVP and a VJP per product."""


class QGTJacobianDense:
    """Marker: the dense QGT S = O_L^T O_L."""


def _qgt_kind(q):
    if q is None or q is QGTAuto or isinstance(q, QGTAuto) or q == "auto":
        return "auto"
    if q is QGTOnTheFly or isinstance(q, QGTOnTheFly) or q == "onthefly":
        return "onthefly"
    if q is QGTJacobianDense or isinstance(q, QGTJacobianDense) or q == "dense":
        return "dense"
    raise ValueError(f"qgt must be QGTAuto, QGTOnTheFly or QGTJacobianDense (or 'auto', "
                     f"'onthefly', 'dense'), not {q!r}")


def _solver_kind(s):
    if s is None or s == "cg":
        return "cg"
    if s == "cholesky" or s is solve_with_fallback:
        return "dense"
    if s is _cholesky or s is _pinv_smooth:
        raise NotImplementedError("SR solves the dense QGT with cholesky_with_fallback; "
                                  "plain cholesky / pinv_smooth are VMC_SR(linear_solver=) "
                                  "choices")
    raise NotImplementedError(f"SR: solver {s!r} is not supported (cg, or the dense "
                              "optimizer.solver.cholesky_with_fallback)")


class SR:
    """Preconditioner ``(vstate, grad, step) -> dp``
    (``netket/optimizer/sr.py:118-216``).

    The QGT form follows ``QGTAuto`` for an RBM (three parameter leaves):
    ``QGTOnTheFly`` with conjugate gradients (``tol``, ``maxiter``; as in NetKet
    with ``solver_restart=False``, CG starts from the previous step's
    solution) unless a dense solver (``optimizer.solver.cholesky_with_fallback``
    or ``"cholesky"``) is given, in which case the dense QGT is
    Cholesky-solved with the pinv_smooth fallback.  ``qgt=QGTJacobianDense``
    always takes the dense form (solved the same way), ``qgt=QGTOnTheFly`` the
    matrix-free one.  ``diag_scale`` and holomorphic SR are not implemented."""

    def __init__(self, qgt=None, solver=None, *, diag_shift=0.01, diag_scale=None,
                 solver_restart=False, holomorphic=None, jac_dtype=torch.float64, tol=1e-5,
                 maxiter=None):
        if diag_scale is not None:
            raise NotImplementedError("SR: diag_scale is not implemented")
        if holomorphic:
            raise NotImplementedError("SR: holomorphic SR is not implemented (real RBM path)")
        kind, skind = _qgt_kind(qgt), _solver_kind(solver)
        if kind == "auto":
            kind = "dense" if skind == "dense" else "onthefly"
        if kind == "onthefly" and skind == "dense":
            raise ValueError("QGTOnTheFly is solved iteratively; a dense solver needs "
                             "QGTJacobianDense")
        self.diag_shift = diag_shift
        self.jac_dtype = jac_dtype
        self.qgt = kind
        self.solver = "cg" if kind == "onthefly" else "cholesky"
        self.tol, self.maxiter, self.solver_restart = tol, maxiter, solver_restart
        self._x0 = None
        self.info = None

    def __call__(self, vstate, grad, step=0):
        c = vstate._cache
        if c is None:
            raise RuntimeError("SR needs expect_and_grad to have run on this state")
        shift = self.diag_shift(step) if callable(self.diag_shift) else self.diag_shift
        if self.qgt == "onthefly":
            x0 = None if self.solver_restart else self._x0
            dp, self.info = sr_update_onthefly(c["t"], c["x"], vstate.N, vstate.M, c["e"],
                                               c["stats_dev"][0:1], shift, x0=x0, tol=self.tol,
                                               maxiter=self.maxiter)
            self._x0 = dp
            return dp
        dp, self.info = sr_update(c["t"], c["x"], vstate.N, vstate.M, c["e"],
                                  c["stats_dev"][0:1], shift, jac_dtype=self.jac_dtype)
        return dp

    def __repr__(self):
        return f"SR(diag_shift={self.diag_shift}, qgt={self.qgt!r}, solver={self.solver!r})"


def identity_preconditioner(vstate, grad, step=0):
    return _flat(grad, vstate.model)


def _cholesky(A, b):
    st = torch.zeros(1, dtype=torch.int32, device=nat.device())
    x = K.cholesky_solve(A, b, st)
    return x, {"status": int(st.item())}


def _pinv_smooth(A, b, rtol=1e-14, rtol_smooth=1e-14):
    return K.pinv_smooth_solve(A, b, rtol, rtol_smooth), None


solver = types.SimpleNamespace(cholesky=_cholesky, cholesky_with_fallback=solve_with_fallback,
                               pinv_smooth=_pinv_smooth)

qgt = types.SimpleNamespace(QGTAuto=QGTAuto, QGTOnTheFly=QGTOnTheFly,
                            QGTJacobianDense=QGTJacobianDense)
