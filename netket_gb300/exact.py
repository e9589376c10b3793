"""Exact diagonalisation (``netket.exact``, ``netket/exact.py:24-131``):
``scipy.sparse.linalg.eigsh`` / ``numpy.linalg.eigh`` on the operator's sparse
or dense matrix, which is assembled from the GPU ``get_conn_padded`` over
every basis state."""
import numpy as np
import scipy.sparse.linalg as spla


def lanczos_ed(operator, *, k=1, compute_eigenvectors=False, matrix_free=False,
               scipy_args=None):
    """The ``k`` lowest eigenvalues (ascending) and, optionally, eigenvectors
    as columns.  ``matrix_free`` hands ARPACK a linear operator (here over the
    assembled sparse matrix) instead of the matrix."""
    H = operator.to_sparse()
    if matrix_free:
        H = spla.LinearOperator(H.shape, matvec=H.__matmul__, dtype=H.dtype)
    args = dict(scipy_args or {})
    args["k"] = k
    args["which"] = "SA"
    if compute_eigenvectors:
        w, v = spla.eigsh(H, return_eigenvectors=True, **args)
        order = np.argsort(w)
        return w[order], v[:, order]
    w = spla.eigsh(H, return_eigenvectors=False, **args)
    return np.sort(w)


def full_ed(operator, *, compute_eigenvectors=False):
    """Every eigenvalue (ascending) and, optionally, the eigenvectors, by dense
    diagonalisation (``netket/exact.py:100-131``)."""
    H = operator.to_dense()
    if compute_eigenvectors:
        return np.linalg.eigh(H)
    return np.linalg.eigvalsh(H)
