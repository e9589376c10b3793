"""Optimisers and the SR preconditioner (``netket.optimizer``).

* ``Sgd(learning_rate)``: ``optax.sgd`` as NetKet wraps it
  (``netket/optimizer/__init__.py:33-60``): ``theta <- theta - lr * update``,
  applied by the ``vmck_sgd`` kernel on the FP64 master parameters.
* ``SR(diag_shift)``: stochastic reconfiguration with the dense QGT
  ``S = O_L^T O_L`` (``netket/optimizer/sr.py:62-216``,
  ``netket/optimizer/qgt/qgt_jacobian_dense.py``) solved by Cholesky with the
  pinv_smooth fallback.
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


class SR:
    """Preconditioner ``(vstate, grad, step) -> dp``.

    ``qgt="dense"`` (default here): the dense QGT solved by Cholesky with the
    pinv_smooth fallback.  ``qgt="onthefly"``: ``QGTOnTheFly`` with conjugate
    gradients (``solver="cg"``, ``tol``, ``maxiter``), NetKet's own default for an
    RBM; as in NetKet (``solver_restart=False``) CG starts from the previous
    step's solution."""

    def __init__(self, diag_shift=0.01, *, jac_dtype=torch.float64, qgt="dense", solver="cholesky",
                 tol=1e-5, maxiter=None, solver_restart=False):
        if qgt not in ("dense", "onthefly"):
            raise ValueError(f"qgt must be 'dense' or 'onthefly', not {qgt!r}")
        self.diag_shift = diag_shift
        self.jac_dtype = jac_dtype
        self.qgt = qgt
        self.solver = "cg" if qgt == "onthefly" else solver
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
