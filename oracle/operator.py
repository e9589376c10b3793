"""Oracle: connected elements of Ising and LocalOperator/Heisenberg
(test infrastructure only).

* ``ising_get_conn_padded`` restates ``IsingJax.get_conn_padded``
  (``netket/operator/_ising/jax.py:82-88, 125-165``).
* ``LocalOperator`` restates the canonicalisation
  (``netket/operator/_local_operator/helpers.py:75-133``), the ``_operators_dict``
  summation (``netket/operator/_local_operator/base.py:135-147``), the packing
  (``netket/operator/_local_operator/compile_helpers.py:29-218, 221-314``) and
  both connected-element kernels: the padded JAX one
  (``netket/operator/_local_operator/jax.py:74-201``) and the flattened numba one
  (``netket/operator/_local_operator/numba.py:132-240``).
* ``Heisenberg`` / ``GraphOperator`` restate ``netket/operator/_heisenberg.py:33-132``
  and ``netket/operator/_graph_operator.py:47-145``.

States are int8 spin values (+1/-1).  Everything is FP64.
"""
import numpy as np
import scipy.sparse as sp

from .hilbert import states_to_local_indices, local_indices_to_states


# ----------------------------------------------------------------------------
# Ising
# ----------------------------------------------------------------------------

def ising_get_conn_padded(x, edges, h, J):
    """Padded connected elements of ``-h sum_i X_i + J sum_<ij> Z_i Z_j``.

    Row 0 is ``x`` with mel ``J * sum_e (2 [x_u == x_v] - 1)``; row ``k`` (1..N)
    is ``x`` with site ``k-1`` flipped and mel ``-h``.  With ``h == 0`` only row 0.
    """
    x = np.asarray(x, dtype=np.int8)
    batch = x.shape[:-1]
    N = x.shape[-1]
    x2 = x.reshape(-1, N)
    e = np.asarray(edges, dtype=np.int64).reshape(-1, 2)
    same = (x2[:, e[:, 0]] == x2[:, e[:, 1]]).astype(np.int64)
    diag = J * (2 * same - 1).sum(axis=-1)
    if h == 0:
        xp = x2[:, None, :].copy()
        mels = diag[:, None].astype(np.float64)
    else:
        K = N + 1
        xp = np.repeat(x2[:, None, :], K, axis=1)
        for k in range(N):
            xp[:, k + 1, k] = -xp[:, k + 1, k]
        mels = np.empty((x2.shape[0], K), dtype=np.float64)
        mels[:, 0] = diag
        mels[:, 1:] = -h
    return xp.reshape(batch + xp.shape[1:]), mels.reshape(batch + mels.shape[1:])


def ising_n_conn(x, edges, h, J):
    _, mels = ising_get_conn_padded(x, edges, h, J)
    n = (0 if h == 0 else x.shape[-1]) + (mels[..., 0] != 0).astype(np.int32)
    return n


# ----------------------------------------------------------------------------
# LocalOperator
# ----------------------------------------------------------------------------

def _reorder(mat, acting_on):
    """Sort ``acting_on`` and permute the matrix's tensor axes to match
    (``helpers.py:149`` ``_reorder_kronecker_product``; first site is the most
    significant digit of the row index)."""
    aon = list(acting_on)
    perm = list(np.argsort(aon, kind="stable"))
    if perm == list(range(len(aon))):
        return np.asarray(mat), tuple(aon)
    k = len(aon)
    t = np.asarray(mat).reshape((2,) * (2 * k))
    t = t.transpose(perm + [k + p for p in perm])
    return t.reshape(2**k, 2**k), tuple(aon[p] for p in perm)


def _number_to_state(number, size):
    # compile_helpers.py:301-314 (spin-1/2: every local size is 2)
    out = np.zeros(size, dtype=np.int64)
    ip, k = number, size - 1
    while ip > 0:
        out[k] = ip % 2
        ip //= 2
        k -= 1
    return out


def _pack_group(ops, cutoff):
    """Tables for a list of (acting_on, matrix) with equal acting size."""
    n_ops = len(ops)
    size = len(ops[0][0])
    R = 2**size
    counts = []
    for _, m in ops:
        mask = np.abs(m) >= cutoff
        np.fill_diagonal(mask, False)
        counts.append(int(mask.sum(axis=1).max()))
    ncmax = max(counts)
    acting_on = np.array([a for a, _ in ops], dtype=np.int64).reshape(n_ops, size)
    diag = np.full((n_ops, R), np.nan)
    mels = np.full((n_ops, R, ncmax), np.nan)
    xprime = np.full((n_ops, R, ncmax, size), -1, dtype=np.int64)
    n_conns = np.zeros((n_ops, R), dtype=np.int64)
    for t, (_, m) in enumerate(ops):
        for r in range(R):
            diag[t, r] = m[r, r]
            c = 0
            for col in range(R):
                if col != r and abs(m[r, col]) > cutoff:
                    mels[t, r, c] = m[r, col]
                    xprime[t, r, c] = _number_to_state(col, size)
                    c += 1
            n_conns[t, r] = c
    nonzero_diag = bool(np.any(np.abs(diag) >= cutoff))
    return dict(acting_on=acting_on, diag_mels=diag, mels=mels, x_prime=xprime,
                n_conns=n_conns, ncmax=ncmax, max_offdiag=counts,
                nonzero_diagonal=nonzero_diag)


class LocalOperator:
    """Sum of k-local spin-1/2 terms (real FP64 matrices)."""

    def __init__(self, N, operators=(), acting_on=(), constant=0.0, mel_cutoff=1e-10):
        self.N = int(N)
        self.constant = float(constant)
        self.mel_cutoff = float(mel_cutoff)
        self._ops = {}
        for op, aon in zip(operators, acting_on):
            m, a = _reorder(np.asarray(op, dtype=np.float64), aon)
            if a in self._ops:
                self._ops[a] = self._ops[a] + m
            else:
                self._ops[a] = m
        self._packed = None

    @property
    def acting_on(self):
        return list(self._ops.keys())

    @property
    def operators(self):
        return list(self._ops.values())

    # -- packing as in pack_internals_jax (compile_helpers.py:174-218)
    def pack(self):
        if self._packed is None:
            items = list(self._ops.items())
            sizes = np.array([len(a) for a, _ in items], dtype=np.int64)
            groups = []
            nonzero = abs(self.constant) >= self.mel_cutoff
            K = 0
            for s in (np.unique(sizes) if len(sizes) else []):
                idx = np.where(sizes == s)[0]
                g = _pack_group([items[i] for i in idx], self.mel_cutoff)
                groups.append(g)
                nonzero = nonzero or g["nonzero_diagonal"]
                K += int(np.sum(g["max_offdiag"]))
            if nonzero:
                K += 1
            self._packed = dict(groups=groups, nonzero_diagonal=bool(nonzero),
                                max_conn_size=int(K))
        return self._packed

    @property
    def max_conn_size(self):
        return self.pack()["max_conn_size"]

    @staticmethod
    def _rows(xi, acting_on):
        sub = xi[acting_on]  # (terms, size)
        size = acting_on.shape[1]
        w = 2 ** np.arange(size - 1, -1, -1)
        return (sub * w).sum(axis=-1)

    def get_conn_padded(self, x):
        """Padded (n, K, N) states and (n, K) mels with JAX-kernel ordering:
        [diagonal] + group-by-acting-size, term, column; entries with
        ``|mel| <= mel_cutoff`` dropped; padding ``(x, 0.0)``."""
        P = self.pack()
        x = np.asarray(x, dtype=np.int8)
        batch = x.shape[:-1]
        x2 = x.reshape(-1, self.N)
        ids = states_to_local_indices(x2).astype(np.int64)
        K = P["max_conn_size"]
        xp = np.repeat(x2[:, None, :], K, axis=1)
        mels = np.zeros((x2.shape[0], K))
        cut = self.mel_cutoff
        for b in range(x2.shape[0]):
            cand = []
            rows = [self._rows(ids[b], g["acting_on"]) for g in P["groups"]]
            if P["nonzero_diagonal"]:
                s = 0.0
                for g, r in zip(P["groups"], rows):
                    gs = 0.0
                    for t in range(len(r)):
                        gs += g["diag_mels"][t, r[t]]
                    s += gs
                cand.append((None, self.constant + s))
            for g, r in zip(P["groups"], rows):
                for t in range(len(r)):
                    nc = g["n_conns"][t, r[t]]
                    for c in range(g["ncmax"]):
                        if c < nc:
                            cand.append(((g["acting_on"][t], g["x_prime"][t, r[t], c]),
                                         g["mels"][t, r[t], c]))
            k = 0
            for change, mel in cand:
                if not abs(mel) > cut:
                    continue
                if k >= K:
                    break
                mels[b, k] = mel
                if change is not None:
                    sites, new_idx = change
                    xp[b, k, sites] = local_indices_to_states(new_idx)
                k += 1
        return xp.reshape(batch + (K, self.N)), mels.reshape(batch + (K,))

    def get_conn_flattened_numba_order(self, x):
        """Per-sample lists in the numba kernel's order (diagonal always kept when
        the operator has a nonzero diagonal; terms in dict order)."""
        P = self.pack()
        x = np.asarray(x, dtype=np.int8).reshape(-1, self.N)
        ids = states_to_local_indices(x).astype(np.int64)
        items = list(self._ops.items())
        out = []
        for b in range(x.shape[0]):
            xs, ms = [], []
            if P["nonzero_diagonal"]:
                d = self.constant
                for a, m in items:
                    r = self._rows(ids[b], np.array([a]))[0]
                    d += m[r, r]
                xs.append(x[b].copy())
                ms.append(d)
            for a, m in items:
                r = self._rows(ids[b], np.array([a]))[0]
                for col in range(m.shape[0]):
                    if col != r and abs(m[r, col]) > self.mel_cutoff:
                        y = x[b].copy()
                        y[list(a)] = local_indices_to_states(_number_to_state(col, len(a)))
                        xs.append(y)
                        ms.append(m[r, col])
            out.append((np.array(xs, dtype=np.int8).reshape(-1, self.N), np.array(ms)))
        return out


def graph_operator(N, graph, site_ops=(), bond_ops=(), bond_ops_colors=()):
    """``GraphOperator`` term order: site ops per node, then bond ops per edge
    (colour-filtered when colours are given)."""
    ops, aon = [], []
    for i in range(graph.n_nodes):
        for so in site_ops:
            ops.append(np.asarray(so, dtype=np.float64))
            aon.append([i])
    if len(bond_ops_colors) > 0:
        for u, v, color in graph.edges(return_color=True):
            for c, bc in enumerate(bond_ops_colors):
                if bc == color:
                    ops.append(np.asarray(bond_ops[c], dtype=np.float64))
                    aon.append([u, v])
    elif len(bond_ops) > 0:
        assert len(bond_ops) == 1
        for u, v in graph.edges():
            ops.append(np.asarray(bond_ops[0], dtype=np.float64))
            aon.append([u, v])
    return LocalOperator(N, ops, aon)


SZSZ = np.array([[1, 0, 0, 0], [0, -1, 0, 0], [0, 0, -1, 0], [0, 0, 0, 1]], dtype=np.float64)
EXCHANGE = np.array([[0, 0, 0, 0], [0, 0, 2, 0], [0, 2, 0, 0], [0, 0, 0, 0]], dtype=np.float64)


def heisenberg(N, graph, J=1.0, sign_rule=None):
    """``J * (SzSz +/- 2 (S+S- + S-S+))`` per bond; sign rule defaults to
    bipartiteness for scalar J and to ``False`` per colour for a J list."""
    if isinstance(J, (list, tuple)):
        if sign_rule is None:
            sign_rule = [False] * len(J)
        bond_ops = [J[i] * (SZSZ - EXCHANGE if sign_rule[i] else SZSZ + EXCHANGE)
                    for i in range(len(J))]
        return graph_operator(N, graph, bond_ops=bond_ops, bond_ops_colors=list(range(len(J))))
    if sign_rule is None:
        sign_rule = graph.is_bipartite()
    bond = J * (SZSZ - EXCHANGE if sign_rule else SZSZ + EXCHANGE)
    return graph_operator(N, graph, bond_ops=[bond])


SIGMAX = np.array([[0.0, 1.0], [1.0, 0.0]])
SIGMAZ = np.array([[1.0, 0.0], [0.0, -1.0]])


def ising_as_local_operator(N, edges, h, J):
    """``IsingBase.to_local_operator`` (``netket/operator/_ising/base.py``): -h X_i
    terms first, then J Z_i Z_j per edge."""
    ops, aon = [], []
    if h != 0:
        for i in range(N):
            ops.append(-h * SIGMAX)
            aon.append([i])
    if J != 0:
        for i, j in edges:
            ops.append(J * np.kron(SIGMAZ, SIGMAZ))
            aon.append([int(i), int(j)])
    return LocalOperator(N, ops, aon)


def to_sparse_from_conn(get_conn, states):
    """Sparse matrix <x|H|x'> over ``states`` built from a padded get_conn."""
    n = len(states)
    index = {s.tobytes(): i for i, s in enumerate(states)}
    xp, mels = get_conn(states)
    rows, cols, vals = [], [], []
    for i in range(n):
        for k in range(mels.shape[1]):
            if mels[i, k] != 0:
                j = index.get(xp[i, k].tobytes())
                if j is None:
                    raise ValueError("connected state outside the basis")
                rows.append(i)
                cols.append(j)
                vals.append(mels[i, k])
    return sp.csr_matrix((vals, (rows, cols)), shape=(n, n))


# ---------------------------------------------------------------- PauliStrings
def pauli_canonicalize(operators, weights):
    """The constructor's reduction (``_pauli_strings/base.py:61-137`` ->
    ``_reduce_pauli_string`` / ``_remove_zero_weights``, ``:564-599``): with
    duplicate strings, the distinct strings in sorted order with summed
    weights; then weights ``isclose`` to 0 are dropped, and an operator left
    empty keeps one identity string of weight 0."""
    ops = np.asarray(list(operators), dtype=str)
    w = np.asarray(weights, dtype=np.float64)
    if len(ops) == 0:
        return ops, w
    uniq, inv = np.unique(ops, return_inverse=True)
    if len(uniq) != len(ops):
        w = np.array([np.sum(w[inv == i]) for i in range(len(uniq))])
        ops = uniq
    keep = ~np.isclose(w, 0)
    if np.any(keep):
        return ops[keep], w[keep]
    return np.array(["I" * len(ops[0])]), np.zeros(1)


def pauli_pack(operators, weights, cutoff=0.0):
    """Flip sets of a list of Pauli strings (``netket/operator/_pauli_strings/
    jax.py:50-105`` grouping, ``137-238`` ordering).

    Each string flips the sites holding X or Y and reads the sign of the sites
    holding Z or Y; a Y contributes a factor -i, absorbed into the weight.
    Strings with the same flip set form one connected element.  Elements are
    ordered by how many strings share them (ascending), then by first
    appearance.  Returns a list of (flip_sites tuple, [(weight, z_sites)])."""
    acting = {}
    for op, w in zip(operators, weights):
        if abs(w) <= cutoff:
            continue
        flip = tuple(sorted(i for i, ch in enumerate(op) if ch in "XY"))
        ny = sum(ch == "Y" for ch in op)
        wt = complex(w) * (-1j) ** ny
        if wt.imag == 0:
            wt = wt.real
        z = sorted(i for i, ch in enumerate(op) if ch in "ZY")
        acting.setdefault(flip, []).append((wt, z))
    by_count = {}
    for flip, rest in acting.items():
        by_count.setdefault(len(rest), []).append((flip, rest))
    return [item for k in sorted(by_count) for item in by_count[k]]


def pauli_get_conn_padded(x, operators, weights, cutoff=1e-10):
    """PauliStringsJax.get_conn_padded on +-1 states: one slot per flip set,
    mel = sum_s w_s prod_{z in s} (-1)^[x_z = -1]; slots with |mel| <= cutoff
    hold (x, 0) (``jax.py:240-269``), for the operator the constructor builds
    from (operators, weights).  Also returns n_conn (nonzero slots)."""
    groups = pauli_pack(*pauli_canonicalize(operators, weights))
    x = np.asarray(x, dtype=np.int8)
    n, N = x.shape
    F = len(groups)
    xp = np.repeat(x[:, None, :], F, axis=1)
    mels = np.zeros((n, F))
    for f, (flip, rest) in enumerate(groups):
        m = np.zeros(n)
        for w, z in rest:
            sgn = np.prod(np.where(x[:, z] < 0, -1.0, 1.0), axis=1) if z else np.ones(n)
            m = m + w * sgn
        keep = np.abs(m) > cutoff
        mels[:, f] = np.where(keep, m, 0.0)
        if flip:
            sub = xp[:, f]
            sub[np.ix_(keep, list(flip))] = -sub[np.ix_(keep, list(flip))]
    return xp, mels, (np.abs(mels) > 0).sum(axis=1)
