"""Exact diagonalisation (``netket.exact.lanczos_ed``, ``netket/exact.py:24-97``):
``scipy.sparse.linalg.eigsh`` on the operator's sparse matrix, which is
assembled from the GPU ``get_conn_padded`` over every basis state."""
import numpy as np
import scipy.sparse.linalg as spla


def lanczos_ed(operator, *, k=1, compute_eigenvectors=False, scipy_args=None):
    H = operator.to_sparse()
    args = dict(k=k, which="SA")
    args.update(scipy_args or {})
    if compute_eigenvectors:
        w, v = spla.eigsh(H, return_eigenvectors=True, **args)
        order = np.argsort(w)
        return w[order], v[:, order]
    w = spla.eigsh(H, return_eigenvectors=False, **args)
    return np.sort(w)
