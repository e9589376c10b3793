"""Oracle: exact diagonalisation and full-sum expectations (test infrastructure only).

* ``lanczos_ed`` restates ``netket/exact.py:24-97``: ``scipy.sparse.linalg.eigsh``
  on the sparse Hamiltonian (here built from the oracle's padded get_conn).
* ``tfim_ground_energy`` is the Jordan-Wigner closed form for the periodic
  transverse-field Ising ring (even-parity sector, antiperiodic momenta), used as
  an independent cross-check of the Lanczos value.
* ``full_sum_energy_and_grad`` is the exact <psi|H|psi>/<psi|psi> and its
  gradient for small N (the idea behind NetKet's FullSumState).
"""
import numpy as np
import scipy.sparse.linalg as spla

from . import rbm
from .hilbert import all_states
from .operator import to_sparse_from_conn


def lanczos_ed(get_conn, N, total_sz=None, k=1):
    states = all_states(N, total_sz)
    H = to_sparse_from_conn(get_conn, states)
    w = spla.eigsh(H, k=k, which="SA", return_eigenvectors=False)
    return np.sort(w)


def tfim_ground_energy(N, J=1.0, h=1.0):
    """Ground energy of ``-h sum X_i + J sum Z_i Z_{i+1}`` on a ring of even N."""
    k = np.pi * (2 * np.arange(N) + 1) / N
    return -np.sum(np.sqrt(J * J + h * h - 2 * abs(J) * h * np.cos(k)))


def full_sum_energy_and_grad(params, get_conn, N, total_sz=None):
    x = all_states(N, total_sz)
    lp = rbm.logpsi(params, x)
    p = np.exp(2 * (lp - lp.max()))
    p /= p.sum()
    eloc = rbm.local_energies(params, x, get_conn)
    E = np.sum(p * eloc)
    O = rbm.jacobian(params, x)
    Obar = p @ O
    grad = 2 * ((O - Obar).T @ (p * (eloc - E)))
    return E, grad
