"""Oracle: spin-1/2 Hilbert space encoding (test infrastructure only).

States are int8 values in {+1, -1} (``netket/hilbert/spin.py:167-172``: new
ordering ``StaticRange(1, -2, 2)``).  Local index 0 <-> +1 and 1 <-> -1
(``netket/utils/static_range.py:148-195``: ``idx = (x - start) / step``).
"""
import itertools

import numpy as np


def states_to_local_indices(x):
    return ((1 - np.asarray(x, dtype=np.int64)) // 2).astype(np.int8)


def local_indices_to_states(idx):
    return (1 - 2 * np.asarray(idx, dtype=np.int64)).astype(np.int8)


def random_state(rng, n_batches, N, total_sz=None):
    """Uniform random states, or for ``total_sz`` a random permutation of the
    fixed number of down spins (``netket/hilbert/random/homogeneous.py:37-72``,
    ``netket/hilbert/random/fock.py:78-101``)."""
    if total_sz is None:
        return local_indices_to_states(rng.integers(0, 2, size=(n_batches, N)))
    n_down = (round(2 * total_sz) - N) // -2
    base = np.zeros((n_batches, N), dtype=np.int64)
    base[:, :n_down] = 1
    idx = rng.permuted(base, axis=1)
    return local_indices_to_states(idx)


def all_states(N, total_sz=None):
    """Every basis state, first site most significant, ``+1`` (index 0) first."""
    idx = np.array(list(itertools.product([0, 1], repeat=N)), dtype=np.int8)
    x = local_indices_to_states(idx)
    if total_sz is not None:
        x = x[x.astype(np.int64).sum(axis=1) == round(2 * total_sz)]
    return x
