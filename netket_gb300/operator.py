"""Hamiltonians of the hot path: ``Ising``, ``LocalOperator``, ``Heisenberg``,
``GraphOperator``, ``PauliStrings`` (``netket.operator`` for spin-1/2).

``get_conn_padded(x)`` follows NetKet's JAX operators (``IsingJax``,
``LocalOperatorJax``): for x (..., N) it returns x' (..., K, N) int8 and
mels (..., K) float64 with ``K = max_conn_size``, computed on the GPU by
``vmck_get_conn_ising`` / ``vmck_get_conn_local``.  Operator tables are packed
on the host once (the work of
``netket/operator/_local_operator/compile_helpers.py:29-218``) and kept
resident on the device.
"""
import ctypes
import types

import numpy as np
import torch

from . import _native as nat
from .graph import Graph


def _as_x(x, N):
    if not isinstance(x, torch.Tensor):
        x = torch.as_tensor(np.asarray(x))
    x = x.to(device=nat.device(), dtype=torch.int8)
    if x.shape[-1] != N:
        raise ValueError(f"last dimension {x.shape[-1]} != N={N}")
    return x.contiguous()


class DiscreteOperator:
    """Shared API of the device operators."""

    is_hermitian = True

    def __init__(self, hilbert):
        self.hilbert = hilbert

    def get_conn_padded(self, x):
        x = _as_x(x, self.hilbert.size)
        batch = x.shape[:-1]
        x2 = x.reshape(-1, self.hilbert.size)
        xp, mels, _ = self._conn(x2)
        K = mels.shape[-1]
        return xp.reshape(*batch, K, self.hilbert.size), mels.reshape(*batch, K)

    def n_conn(self, x):
        x = _as_x(x, self.hilbert.size)
        _, _, n = self._conn(x.reshape(-1, self.hilbert.size))
        return n.reshape(x.shape[:-1])

    def to_sparse(self):
        import scipy.sparse as sp
        states = self.hilbert.all_states()
        xp, mels = self.get_conn_padded(states)
        n, K, N = xp.shape
        w = torch.tensor([1 << (N - 1 - i) for i in range(N)], dtype=torch.int64,
                         device=states.device)
        code_x = (((1 - states.to(torch.int64)) // 2) * w).sum(-1)
        code_xp = (((1 - xp.to(torch.int64)) // 2) * w).sum(-1)
        order = torch.argsort(code_x)
        pos = torch.searchsorted(code_x[order], code_xp.reshape(-1))
        pos = order[pos.clamp(max=n - 1)].reshape(n, K)
        m = mels.cpu().numpy()
        cols = pos.cpu().numpy()
        rows = np.repeat(np.arange(n), K)
        keep = m.reshape(-1) != 0
        return sp.csr_matrix((m.reshape(-1)[keep], (rows[keep], cols.reshape(-1)[keep])),
                             shape=(n, n))

    def __pow__(self, power):
        """``_abstract_operator.py:157-171``: repeated ``@`` for power >= 1."""
        if not isinstance(power, int) or power < 0:
            return NotImplemented
        if power == 0:
            raise NotImplementedError(f"__pow__(0) (identity) is not implemented for "
                                      f"{type(self).__name__}. Use the identity constructor "
                                      "of your operator type directly.")
        result = self
        for _ in range(power - 1):
            result = result @ self
        return result

    def to_dense(self):
        return self.to_sparse().toarray()


class Ising(DiscreteOperator):
    """``-h sum_i X_i + J sum_<ij> Z_i Z_j`` (``netket/operator/_ising/jax.py``)."""

    def __init__(self, hilbert, graph, h, J=1.0, dtype=None):
        _check_real_dtype(dtype, "Ising")
        super().__init__(hilbert)
        if hasattr(graph, "edges"):
            edges = np.asarray(graph.edges(), dtype=np.int64).reshape(-1, 2)
        else:
            edges = np.asarray(graph, dtype=np.int64).reshape(-1, 2)
        self.edges = edges
        self.h = float(h)
        self.J = float(J)
        self._dev = {}

    @property
    def max_conn_size(self):
        return self.hilbert.size + 1

    def _edges_dev(self):
        d = torch.cuda.current_device()
        if d not in self._dev:
            self._dev[d] = torch.as_tensor(self.edges.astype(np.int32), device=nat.device())
        return self._dev[d]

    def _conn(self, x):
        n, N = x.shape
        K = 1 if self.h == 0 else N + 1
        xp = torch.empty((n, K, N), dtype=torch.int8, device=x.device)
        mels = torch.empty((n, K), dtype=torch.float64, device=x.device)
        nc = torch.empty((n,), dtype=torch.int32, device=x.device)
        e = self._edges_dev()
        nat.check(nat.lib().vmck_get_conn_ising(nat.stream(), nat.ptr(x), n, N, nat.ptr(e),
                                                len(self.edges), self.h, self.J,
                                                int(self.h == 0), nat.ptr(xp), nat.ptr(mels),
                                                nat.ptr(nc)))
        return xp, mels, nc

    # algebra: NetKet sums an Ising with other operators lazily (SumOperator,
    # netket/operator/_abstract_operator.py:117-152); here the sum is the
    # concrete LocalOperator of the same matrix, and a scalar multiple stays an
    # Ising (h and J scaled) so it keeps the Ising kernels.
    def __mul__(self, s):
        if isinstance(s, DiscreteOperator):
            return self.to_local_operator() @ _as_local(s)
        if not np.isscalar(s):
            return NotImplemented
        if np.iscomplexobj(np.asarray(s)) and np.imag(s) != 0:
            raise TypeError("Ising: complex coefficients are not supported on this path")
        s = float(np.real(s))
        return Ising(self.hilbert, self.edges, self.h * s, self.J * s)

    def __rmul__(self, s):
        if not np.isscalar(s):
            return NotImplemented
        return self.__mul__(s)

    def __truediv__(self, s):
        if not np.isscalar(s):
            raise TypeError("Only division by a scalar number is supported.")
        if s == 0:
            raise ValueError("Dividing by 0")
        return self.__mul__(1.0 / s)

    def __neg__(self):
        return self * -1.0

    def __add__(self, other):
        if isinstance(other, (Ising, LocalOperator)) or np.isscalar(other):
            return self.to_local_operator() + _as_local(other)
        return NotImplemented

    def __radd__(self, other):
        if isinstance(other, (Ising, LocalOperator)) or np.isscalar(other):
            return _as_local(other) + self.to_local_operator()
        return NotImplemented

    def __sub__(self, other):
        return self + (-other)

    def __rsub__(self, other):
        return other + (-self)

    def __matmul__(self, other):
        if isinstance(other, (Ising, LocalOperator)):
            return self.to_local_operator() @ _as_local(other)
        return NotImplemented

    def __rmatmul__(self, other):
        if isinstance(other, LocalOperator):
            return other @ self.to_local_operator()
        return NotImplemented

    def to_local_operator(self):
        """``IsingBase.to_local_operator``: -h X_i terms, then J Z_i Z_j per edge."""
        ops, aon = [], []
        if self.h != 0:
            for i in range(self.hilbert.size):
                ops.append(-self.h * SIGMAX)
                aon.append([i])
        if self.J != 0:
            for i, j in self.edges:
                ops.append(self.J * np.kron(SIGMAZ, SIGMAZ))
                aon.append([int(i), int(j)])
        return LocalOperator(self.hilbert, ops, aon)

    def __repr__(self):
        return f"Ising(J={self.J}, h={self.h}; dim={self.hilbert.size})"


SIGMAX = np.array([[0.0, 1.0], [1.0, 0.0]])
SIGMAZ = np.array([[1.0, 0.0], [0.0, -1.0]])
SZSZ = np.diag([1.0, -1.0, -1.0, 1.0])
EXCHANGE = np.array([[0, 0, 0, 0], [0, 0, 2, 0], [0, 2, 0, 0], [0, 0, 0, 0]], dtype=np.float64)


def _embed(mat, sites, union):
    """``mat`` on ``sites`` (sorted) as an operator on ``union`` (sorted, a
    superset): identity on the other sites, first site the leading digit."""
    sites = list(sites)
    others = [u for u in union if u not in sites]
    k, u = len(sites), len(union)
    full = np.kron(np.asarray(mat, dtype=np.float64), np.eye(2 ** len(others)))
    order = sites + others
    perm = [order.index(site) for site in union]
    t = full.reshape((2,) * (2 * u)).transpose(perm + [u + p for p in perm])
    return t.reshape(2 ** u, 2 ** u)


def _sort_sites(mat, sites):
    """Sort the sites of a k-local matrix, permuting its tensor factors
    (first site = most significant digit of the row index)."""
    sites = [int(s) for s in sites]
    if len(set(sites)) != len(sites):
        raise ValueError(f"operator acts on duplicated sites {sites}")
    order = sorted(range(len(sites)), key=lambda q: sites[q])
    if order == list(range(len(sites))):
        return np.array(mat, dtype=np.float64), tuple(sites)
    k = len(sites)
    t = np.asarray(mat, dtype=np.float64).reshape((2,) * (2 * k))
    t = np.transpose(t, order + [k + q for q in order])
    return t.reshape(2**k, 2**k), tuple(sites[q] for q in order)


def _real_matrix(op):
    """A term's matrix as float64; imaginary matrix elements are refused rather
    than dropped (the path's operators are real)."""
    a = np.asarray(op)
    if np.iscomplexobj(a):
        if np.any(a.imag != 0):
            raise TypeError("LocalOperator: complex matrix elements are not supported on this "
                            "path (real operators only)")
        a = a.real
    return np.asarray(a, dtype=np.float64)


def _real_scalar(c, name):
    if np.iscomplexobj(np.asarray(c)):
        if np.imag(c) != 0:
            raise TypeError(f"LocalOperator: a complex {name} is not supported on this path")
        c = np.real(c)
    return float(c)


def _as_local(op):
    return op.to_local_operator() if isinstance(op, Ising) else op


class LocalOperator(DiscreteOperator):
    """Sum of k-local spin-1/2 terms (k <= 4), NetKet's ``LocalOperator``."""

    def __init__(self, hilbert, operators=(), acting_on=(), constant=0.0, dtype=None,
                 mel_cutoff=1e-10):
        _check_real_dtype(dtype, "LocalOperator")
        super().__init__(hilbert)
        self.constant = _real_scalar(constant, "constant")
        self.mel_cutoff = float(mel_cutoff)
        self._terms = {}
        if len(acting_on) and np.isscalar(acting_on[0]):
            operators, acting_on = [operators], [acting_on]
        for op, aon in zip(operators, acting_on):
            self._add(_real_matrix(op), aon)
        self._tables = None
        self._dev = {}

    def _add(self, mat, aon):
        if any(a < 0 or a >= self.hilbert.size for a in aon):
            raise ValueError("An operator acts on an invalid set of sites.")
        if mat.shape != (2 ** len(aon), 2 ** len(aon)):
            raise ValueError(f"matrix shape {mat.shape} does not match sites {list(aon)}")
        m, key = _sort_sites(mat, aon)
        self._terms[key] = self._terms[key] + m if key in self._terms else m
        self._herm = None
        self._tables = None
        self._dev = {}

    @property
    def acting_on(self):
        return [list(k) for k in self._terms]

    @property
    def operators(self):
        return list(self._terms.values())

    @property
    def n_operators(self):
        return len(self._terms)

    @property
    def is_hermitian(self):
        """Every term is a symmetric (real) matrix (cached until a term is added)."""
        if getattr(self, "_herm", None) is None:
            self._herm = all(np.allclose(m, m.T) for m in self._terms.values())
        return self._herm

    def to_pauli_strings(self):
        """The same operator as ``PauliStrings`` (``netket/operator/_local_operator/
        convert.py:157-209``): every term projected on the Pauli basis of its
        sites (``itertools.product("IXYZ")`` order, first character on the
        term's first site), weight ``Tr(P A) / 2^k``, the constant as the
        identity string, then the PauliStrings constructor's reduction.  The
        terms are real symmetric, so the strings with an odd number of Y carry
        only rounding and are dropped (the reference drops them in the same
        reduction)."""
        import itertools
        N = self.hilbert.size
        basis = {"I": np.eye(2), "X": np.array([[0.0, 1.0], [1.0, 0.0]]),
                 "Y": np.array([[0.0, -1.0j], [1.0j, 0.0]]),
                 "Z": np.array([[1.0, 0.0], [0.0, -1.0]])}
        strings, weights = [], []
        for aon, m in self._terms.items():
            k = len(aon)
            for chars in itertools.product("IXYZ", repeat=k):
                P = basis[chars[0]]
                for c in chars[1:]:
                    P = np.kron(P, basis[c])
                w = np.trace(P @ m) / 2 ** k
                if w == 0:
                    continue
                if chars.count("Y") % 2:
                    if not np.isclose(w, 0):
                        raise TypeError("to_pauli_strings: the operator is not real")
                    continue
                s = ["I"] * N
                for site, c in zip(aon, chars):
                    s[site] = c
                strings.append("".join(s))
                weights.append(float(np.real(w)))
        if abs(self.constant) > 1e-13:
            strings.append("I" * N)
            weights.append(self.constant)
        return PauliStrings(self.hilbert, strings, weights)

    def copy(self):
        new = LocalOperator(self.hilbert, constant=self.constant, mel_cutoff=self.mel_cutoff)
        new._terms = {k: v.copy() for k, v in self._terms.items()}
        return new

    def __add__(self, other):
        """``_local_operator/base.py:296-332``: operators on another Hilbert
        space do not add; the sum keeps the smaller ``mel_cutoff``."""
        if isinstance(other, LocalOperator):
            if other.hilbert != self.hilbert:
                return NotImplemented
            new = self.copy()
            new.mel_cutoff = min(self.mel_cutoff, other.mel_cutoff)
            for k, v in other._terms.items():
                new._add(v, k)
            new.constant += other.constant
            return new
        if np.isscalar(other):
            new = self.copy()
            new.constant += float(other)
            return new
        return NotImplemented

    __radd__ = __add__

    def __rsub__(self, other):
        return other + (-self)

    def __truediv__(self, other):
        if not np.isscalar(other):
            raise TypeError("Only division by a scalar number is supported.")
        if other == 0:
            raise ValueError("Dividing by 0")
        return self.__mul__(1.0 / other)

    def transpose(self, *, concrete=False):
        """Every term's matrix transposed (``_local_operator/base.py:263-271``;
        returned concrete whatever ``concrete`` says: there are no lazy wrappers
        here)."""
        new = self.copy()
        new._terms = {k: np.ascontiguousarray(v.T) for k, v in self._terms.items()}
        return new

    def conjugate(self, *, concrete=False):
        return self.copy()  # real matrix elements

    def conj(self, *, concrete=False):
        return self.conjugate(concrete=concrete)

    @property
    def T(self):
        return self.transpose()

    @property
    def H(self):
        """The adjoint: the operator itself when hermitian, else its transpose
        (real matrix elements)."""
        return self if self.is_hermitian else self.transpose(concrete=True)

    def __mul__(self, s):
        if isinstance(s, LocalOperator):
            return self @ s
        if not np.isscalar(s):
            return NotImplemented
        new = LocalOperator(self.hilbert, constant=self.constant * s, mel_cutoff=self.mel_cutoff)
        # a scalar at or below mel_cutoff clears the terms (local_operator/base.py:356-376)
        new._terms = {} if abs(s) <= self.mel_cutoff else {k: v * s for k, v in self._terms.items()}
        return new

    def __rmul__(self, s):
        if not np.isscalar(s):
            return NotImplemented
        return self.__mul__(s)

    def __matmul__(self, other):
        """Operator product (``netket/operator/_local_operator/base.py:392-440``):
        (a + sum_i A_i)(b + sum_j B_j) = b (a + sum_i A_i) + a sum_j B_j +
        sum_ij A_i B_j, terms added in that order (equal supports merge), each
        product on the sorted union of its two supports (at most 4 sites)."""
        if not isinstance(other, LocalOperator):
            return NotImplemented
        if other.hilbert != self.hilbert:
            raise ValueError("Can only multiply operators on identical hilbert spaces")
        a, b = self.constant, other.constant
        cut = min(self.mel_cutoff, other.mel_cutoff)
        A, B = list(self._terms.items()), list(other._terms.items())
        new = self * b
        new.mel_cutoff = cut
        if abs(a) > cut:
            for k, v in B:
                new._add(a * v, k)
        for ka, va in A:
            for kb, vb in B:
                union = sorted(set(ka) | set(kb))
                if len(union) > 4:
                    raise NotImplementedError("terms acting on more than 4 sites are not "
                                              "supported")
                new._add(_embed(va, ka, union) @ _embed(vb, kb, union), union)
        new._tables, new._dev = None, {}
        return new

    def __neg__(self):
        return self * -1.0

    def __sub__(self, other):
        return self + (-other)

    # ---------------------------------------------------------------- packing
    def _pack(self):
        """Device tables in JAX-packer order: terms grouped by acting size
        (ascending), insertion order within a group."""
        if self._tables is not None:
            return self._tables
        items = list(self._terms.items())
        sizes = sorted({len(k) for k, _ in items})
        ordered = [(k, m) for s in sizes for (k, m) in items if len(k) == s]
        group_end, acc = [], 0
        for s in sizes:
            acc += sum(1 for k, _ in items if len(k) == s)
            group_end.append(acc)
        T = len(ordered)
        S = max(sizes) if sizes else 1
        if S > 4:
            raise NotImplementedError("terms acting on more than 4 sites are not supported")
        R = 2**S
        cut = self.mel_cutoff
        per_row = []
        K = 0
        nonzero_diag = abs(self.constant) >= cut
        for k, m in ordered:
            off = np.abs(m) > cut
            np.fill_diagonal(off, False)
            per_row.append(off)
            kept = np.abs(m) >= cut
            np.fill_diagonal(kept, False)
            K += int(kept.sum(axis=1).max())
            nonzero_diag = nonzero_diag or bool(np.any(np.abs(np.diag(m)) >= cut))
        C = max([int(o.sum(axis=1).max()) for o in per_row], default=0)
        if nonzero_diag:
            K += 1
        acting_on = np.full((T, S), -1, dtype=np.int32)
        acting_size = np.zeros(T, dtype=np.int32)
        diag = np.zeros((T, R))
        n_conns = np.zeros((T, R), dtype=np.int32)
        mels = np.zeros((T, R, max(C, 1)))
        xprime = np.zeros((T, R, max(C, 1), S), dtype=np.int8)
        for t, ((key, m), off) in enumerate(zip(ordered, per_row)):
            sz = len(key)
            acting_on[t, :sz] = key
            acting_size[t] = sz
            for r in range(2**sz):
                diag[t, r] = m[r, r]
                cols = np.flatnonzero(off[r])
                n_conns[t, r] = len(cols)
                for c, col in enumerate(cols):
                    mels[t, r, c] = m[r, col]
                    bits = [(col >> (sz - 1 - q)) & 1 for q in range(sz)]
                    xprime[t, r, c, :sz] = [1 - 2 * b for b in bits]
        self._tables = dict(T=T, S=S, R=R, C=max(C, 1), K=K, nonzero_diag=bool(nonzero_diag),
                            acting_on=acting_on, acting_size=acting_size,
                            group_end=np.array(group_end, dtype=np.int32), diag=diag,
                            n_conns=n_conns, mels=mels, xprime=xprime)
        return self._tables

    @property
    def max_conn_size(self):
        return self._pack()["K"]

    def device_struct(self):
        """(ctypes ``vmck_local_op``, tensors kept alive) on the current device."""
        d = torch.cuda.current_device()
        if d not in self._dev:
            tb = self._pack()
            dev = nat.device()
            keep = {k: torch.as_tensor(np.ascontiguousarray(tb[k]), device=dev)
                    for k in ("acting_on", "acting_size", "group_end", "diag", "n_conns", "mels",
                              "xprime")}
            st = nat.LocalOpStruct(
                n_sites=self.hilbert.size, n_terms=tb["T"], max_sites=tb["S"], max_rows=tb["R"],
                max_conns=tb["C"], max_conn_size=tb["K"], nonzero_diagonal=int(tb["nonzero_diag"]),
                n_groups=len(tb["group_end"]), constant=self.constant, mel_cutoff=self.mel_cutoff,
                acting_on=keep["acting_on"].data_ptr(), acting_size=keep["acting_size"].data_ptr(),
                group_end=keep["group_end"].data_ptr(), diag_mels=keep["diag"].data_ptr(),
                n_conns=keep["n_conns"].data_ptr(), mels=keep["mels"].data_ptr(),
                x_prime=keep["xprime"].data_ptr())
            self._dev[d] = (st, keep)
        return self._dev[d][0]

    def _conn(self, x):
        n, N = x.shape
        st = self.device_struct()
        K = st.max_conn_size
        xp = torch.empty((n, K, N), dtype=torch.int8, device=x.device)
        mels = torch.empty((n, K), dtype=torch.float64, device=x.device)
        nc = torch.empty((n,), dtype=torch.int32, device=x.device)
        if K == 0:
            return xp, mels, nc.zero_()
        nat.check(nat.lib().vmck_get_conn_local(nat.stream(), ctypes.byref(st), nat.ptr(x), n,
                                                nat.ptr(xp), nat.ptr(mels), nat.ptr(nc)))
        return xp, mels, nc

    def __repr__(self):
        return (f"LocalOperator(dim={self.hilbert.size}, #acting_on={len(self._terms)} "
                f"locations, constant={self.constant})")


def _pauli_mul_table():
    """(a, b) -> (c, f) with a b = f c for single-site Pauli matrices."""
    t = {}
    for p in "IXYZ":
        t["I", p] = (p, 1 + 0j)
        t[p, "I"] = (p, 1 + 0j)
        t[p, p] = ("I", 1 + 0j)
    for a, b, c in (("X", "Y", "Z"), ("Y", "Z", "X"), ("Z", "X", "Y")):
        t[a, b] = (c, 1j)
        t[b, a] = (c, -1j)
    return t


_PAULI_MUL = _pauli_mul_table()


def _reduce_strings(ops, w, n_sites):
    """The PauliStrings reduction (``_pauli_strings/base.py:564-599``):
    duplicate strings summed in sorted string order, weights within
    ``np.isclose(., 0)`` of zero dropped (all dropped: the identity with 0)."""
    uniq, inv = np.unique(ops, return_inverse=True)
    if len(uniq) != len(ops):
        w = np.array([np.sum(w[inv == i]) for i in range(len(uniq))], dtype=w.dtype)
        ops = uniq
    keep = ~np.isclose(w, 0)
    if np.any(keep):
        return ops[keep], w[keep]
    return np.array(["I" * n_sites]), np.zeros(1, dtype=w.dtype)


class PauliStrings(DiscreteOperator):
    """Sum of weighted Pauli strings (``netket/operator/_pauli_strings``), e.g.
    ``PauliStrings(hi, ["XXI", "ZZI"], [0.5, 1.0])``; character k of a string
    acts on site k.  Strings that flip the same sites share one connected
    element, ordered as PauliStringsJax orders them
    (``_pauli_strings/jax.py:137-238``).  Real matrix elements only: every
    string needs an even number of Y (a real weight times (-i)^#Y)."""

    def __init__(self, hilbert, operators=None, weights=None, *, cutoff=1.0e-10, dtype=None):
        super().__init__(hilbert)
        if operators is None:
            operators = []
        if isinstance(operators, str):
            operators = [operators]
        operators = [str(o) for o in operators]
        if weights is None:
            weights = [1.0] * len(operators)
        elif np.isscalar(weights):
            weights = [weights] * len(operators)
        weights = list(weights)
        if len(weights) != len(operators):
            raise ValueError("weights and operators must have the same length")
        for o in operators:
            if len(o) != hilbert.size or any(ch not in "XYZI" for ch in o):
                raise ValueError(f"invalid Pauli string {o!r} for {hilbert.size} sites")
        if any(np.iscomplexobj(np.asarray(w)) and np.imag(w) != 0 for w in weights):
            raise TypeError("PauliStrings: complex weights are not supported on this path")
        if any(o.count("Y") % 2 for o in operators):
            raise TypeError("PauliStrings: a string with an odd number of Y has imaginary "
                            "matrix elements, not supported on this path")
        ops = np.asarray(operators, dtype=str)
        w = np.asarray([float(np.real(v)) for v in weights], dtype=np.float64)
        if len(ops):
            ops, w = _reduce_strings(ops, w, hilbert.size)
        self.operators = [str(o) for o in ops]
        self.weights = [float(v) for v in w]
        self.cutoff = float(cutoff)
        self._tables = None
        self._dev = {}

    # ------------------------------------------------------------ algebra
    # (netket/operator/_pauli_strings/base.py:330-470): + concatenates and reduces
    # as the constructor does; a scalar adds the identity string; * scales the
    # weights (no reduction); @ multiplies string by string.
    def __matmul__(self, other):
        """Product of two sums of strings (``_pauli_strings/base.py:330-371,
        522-660``): every pair (self's string major), site by site with
        XY = iZ, YZ = iX, ZX = iY (reversed order: -i), weight w1 w2 times the
        phase, then the constructor's reduction.  The reference switches to
        complex weights when some product string has an odd number of Y; the
        result is returned here when every reduced weight is real (imaginary
        parts that cancel included) and refused otherwise."""
        if not isinstance(other, PauliStrings):
            return NotImplemented
        if other.hilbert != self.hilbert:
            raise ValueError(f"Can only multiply identical hilbert spaces (got A@B, "
                             f"A={self.hilbert}, B={other.hilbert})")
        ops, ws = [], []
        for o1, w1 in zip(self.operators, self.weights):
            for o2, w2 in zip(other.operators, other.weights):
                phase = 1 + 0j
                chars = []
                for a, b in zip(o1, o2):
                    c, f = _PAULI_MUL[a, b]
                    chars.append(c)
                    phase *= f
                ops.append("".join(chars))
                ws.append((w1 * w2) * phase)
        ops, w = _reduce_strings(np.asarray(ops, dtype=str), np.asarray(ws, np.complex128),
                                 self.hilbert.size)
        if np.any(np.imag(w) != 0):
            raise TypeError("PauliStrings @ PauliStrings gives complex weights here; they "
                            "are not supported on this path")
        return PauliStrings(self.hilbert, [str(o) for o in ops], np.real(w),
                            cutoff=min(self.cutoff, other.cutoff))

    def _scaled(self, c):
        new = object.__new__(PauliStrings)
        DiscreteOperator.__init__(new, self.hilbert)
        new.operators = list(self.operators)
        new.weights = [w * float(c) for w in self.weights]
        new.cutoff = self.cutoff
        new._tables, new._dev = None, {}
        return new

    def __add__(self, other):
        if isinstance(other, PauliStrings):
            if other.hilbert != self.hilbert:
                raise ValueError(f"Can only add identical hilbert spaces (got A+B, "
                                 f"A={self.hilbert}, B={other.hilbert})")
            return PauliStrings(self.hilbert, self.operators + other.operators,
                                self.weights + other.weights,
                                cutoff=min(self.cutoff, other.cutoff))
        if np.isscalar(other):
            if other == 0:
                return self._scaled(1.0)
            return self + PauliStrings(self.hilbert, "I" * self.hilbert.size, float(other),
                                       cutoff=self.cutoff)
        return NotImplemented

    def __radd__(self, other):
        if np.isscalar(other):
            return self.__add__(other)
        return NotImplemented

    def __mul__(self, other):
        if isinstance(other, DiscreteOperator):
            raise TypeError("To multiply operators use the matrix`@` multiplication operator "
                            "`@` instead of the element-wise multiplication operator `*`.")
        if np.isscalar(other):
            if np.iscomplexobj(np.asarray(other)) and np.imag(other) != 0:
                raise TypeError("PauliStrings: complex weights are not supported on this path")
            return self._scaled(float(np.real(other)))
        return NotImplemented

    __rmul__ = __mul__

    def __neg__(self):
        return self._scaled(-1.0)

    def __sub__(self, other):
        return self + (-other)

    def __rsub__(self, other):
        return other + (-self)

    def _pack(self):
        if self._tables is not None:
            return self._tables
        N = self.hilbert.size
        W = (N + 31) // 32
        acting = {}
        for op, w in zip(self.operators, self.weights):
            if abs(w) <= self.cutoff:
                continue
            flip = tuple(i for i, ch in enumerate(op) if ch in "XY")
            wt = w * (-1.0) ** (op.count("Y") // 2)  # (-i)^#Y for an even #Y
            z = [i for i, ch in enumerate(op) if ch in "ZY"]
            acting.setdefault(flip, []).append((wt, z))
        by_count = {}
        for flip, rest in acting.items():
            by_count.setdefault(len(rest), []).append((flip, rest))
        slots = [item for k in sorted(by_count) for item in by_count[k]]

        def mask(sites):
            m = np.zeros(W, dtype=np.uint32)
            for i in sites:
                m[i // 32] |= np.uint32(1 << (i % 32))
            return m

        F = len(slots)
        flip_mask = np.zeros((max(F, 1), W), dtype=np.uint32)
        flip_offset, flip_site, string_offset, z_mask, weight = [0], [], [0], [], []
        for f, (flip, rest) in enumerate(slots):
            flip_mask[f] = mask(flip)
            flip_site.extend(flip)
            flip_offset.append(len(flip_site))
            for wt, z in rest:
                z_mask.append(mask(z))
                weight.append(wt)
            string_offset.append(len(weight))
        self._tables = dict(
            N=N, W=W, F=F, S=len(weight), flip_mask=flip_mask,
            flip_offset=np.array(flip_offset, dtype=np.int32),
            flip_site=np.array(flip_site + [0], dtype=np.int32),
            string_offset=np.array(string_offset, dtype=np.int32),
            z_mask=np.array(z_mask, dtype=np.uint32).reshape(-1, W) if z_mask else
            np.zeros((1, W), dtype=np.uint32),
            weight=np.array(weight + [0.0], dtype=np.float64))
        return self._tables

    @property
    def max_conn_size(self):
        return self._pack()["F"]

    def device_struct(self):
        d = torch.cuda.current_device()
        if d not in self._dev:
            tb = self._pack()
            dev = nat.device()
            keep = {}
            for k in ("flip_mask", "z_mask"):
                keep[k] = torch.as_tensor(tb[k].view(np.int32), device=dev).contiguous()
            for k in ("flip_offset", "flip_site", "string_offset", "weight"):
                keep[k] = torch.as_tensor(tb[k], device=dev).contiguous()
            st = nat.PauliStringsStruct(
                n_sites=tb["N"], n_words=tb["W"], n_flips=tb["F"], n_strings=tb["S"],
                cutoff=self.cutoff, flip_mask=keep["flip_mask"].data_ptr(),
                flip_offset=keep["flip_offset"].data_ptr(), flip_site=keep["flip_site"].data_ptr(),
                string_offset=keep["string_offset"].data_ptr(), z_mask=keep["z_mask"].data_ptr(),
                weight=keep["weight"].data_ptr())
            self._dev[d] = (st, keep)
        return self._dev[d][0]

    def _conn(self, x):
        n, N = x.shape
        st = self.device_struct()
        F = st.n_flips
        xp = torch.empty((n, F, N), dtype=torch.int8, device=x.device)
        mels = torch.empty((n, F), dtype=torch.float64, device=x.device)
        nc = torch.empty((n,), dtype=torch.int32, device=x.device)
        nat.check(nat.lib().vmck_get_conn_pauli(nat.stream(), ctypes.byref(st), nat.ptr(x), n,
                                                nat.ptr(xp), nat.ptr(mels), nat.ptr(nc)))
        return xp, mels, nc

    def __repr__(self):
        return f"PauliStrings(hilbert={self.hilbert}, n_strings={len(self.operators)})"


def check_acting_on_subspace(acting_on_subspace, hilbert, graph):
    """Graph node -> Hilbert site map (``netket/operator/_graph_operator.py:29-44``):
    None is the identity, an int ``start`` maps node i to start + i, a list is
    the map itself (one entry per node)."""
    if acting_on_subspace is None:
        return list(range(hilbert.size))
    if isinstance(acting_on_subspace, (int, np.integer)) and not isinstance(acting_on_subspace,
                                                                            bool):
        return [int(acting_on_subspace) + i for i in range(graph.n_nodes)]
    if isinstance(acting_on_subspace, list):
        if len(acting_on_subspace) != graph.n_nodes:
            raise ValueError("acting_on_subspace must be a list of length graph.n_nodes")
        return acting_on_subspace
    raise TypeError("acting_on_subspace must be a list or single integer")


def _check_real_dtype(dtype, name):
    if dtype is not None and np.issubdtype(np.dtype(dtype), np.complexfloating):
        raise TypeError(f"{name}: complex matrix elements are not supported on this path")


def GraphOperator(hilbert, graph, site_ops=(), bond_ops=(), bond_ops_colors=(), dtype=None, *,
                  acting_on_subspace=None):
    """Sum of site operators on every node and bond operators on every edge
    (coloured edges select their operator), NetKet's term order
    (``netket/operator/_graph_operator.py:47-145``); node i acts on site
    ``acting_on_subspace[i]``."""
    _check_real_dtype(dtype, "GraphOperator")
    sites = check_acting_on_subspace(acting_on_subspace, hilbert, graph)
    if len(site_ops) == 0 and len(bond_ops) == 0:
        raise ValueError("Must input at least site_ops or bond_ops.")
    ops, aon = [], []
    for i in range(graph.n_nodes):
        for so in site_ops:
            ops.append(so)
            aon.append([sites[i]])
    if len(bond_ops_colors) > 0:
        if len(bond_ops) != len(bond_ops_colors):
            raise ValueError("The sizes of bond_ops and bond_ops_colors do not match.")
        for u, v, color in graph.edges(return_color=True):
            for c, bc in enumerate(bond_ops_colors):
                if bc == color:
                    ops.append(bond_ops[c])
                    aon.append([sites[u], sites[v]])
    elif len(bond_ops) > 0:
        if len(bond_ops) != 1:
            raise ValueError("without colours exactly one bond operator is expected")
        for u, v in graph.edges():
            ops.append(bond_ops[0])
            aon.append([sites[u], sites[v]])
    return LocalOperator(hilbert, ops, aon)


def Heisenberg(hilbert, graph, J=1.0, sign_rule=None, dtype=None, *, acting_on_subspace=None):
    """``J (Sz Sz +/- 2 (S+S- + S-S+))`` per bond (``netket/operator/_heisenberg.py:31-132``);
    the minus sign applies Marshall's sign rule (default: bipartite graph for a
    scalar J, ``False`` per colour for a J list; refused on a graph, or a
    colour's subgraph, that is not bipartite)."""
    if isinstance(J, (list, tuple)):
        if len(J) != max(graph.edge_colors) + 1:
            raise ValueError("one coupling per edge colour is expected")
        if sign_rule is None:
            sign_rule = [False] * len(J)
        else:
            if len(sign_rule) != len(J):
                raise ValueError("one sign_rule entry per coupling is expected")
            for i in range(len(J)):
                if sign_rule[i] and not Graph(graph.edges(filter_color=i)).is_bipartite():
                    raise ValueError("sign_rule=True specified for a non-bipartite lattice")
        bond_ops = [J[i] * (SZSZ - EXCHANGE if sign_rule[i] else SZSZ + EXCHANGE)
                    for i in range(len(J))]
        return GraphOperator(hilbert, graph, bond_ops=bond_ops, bond_ops_colors=list(range(len(J))),
                             dtype=dtype, acting_on_subspace=acting_on_subspace)
    if sign_rule is None:
        sign_rule = graph.is_bipartite()
    elif sign_rule and not graph.is_bipartite():
        raise ValueError("sign_rule=True specified for a non-bipartite lattice")
    return GraphOperator(hilbert, graph,
                         bond_ops=[J * (SZSZ - EXCHANGE if sign_rule else SZSZ + EXCHANGE)],
                         dtype=dtype, acting_on_subspace=acting_on_subspace)


# -------------------------------------------------------------------- spin
def _spin_site(hilbert, site, mat):
    return LocalOperator(hilbert, [np.asarray(mat, dtype=np.float64)], [[int(site)]])


def _identity(hilbert, dtype=None):
    """The identity (``netket/operator/spin.py:29-45``)."""
    return LocalOperator(hilbert, constant=1.0)


def _sigmax(hilbert, site, dtype=None):
    """Pauli X on ``site`` (``netket/operator/spin.py:48-78``)."""
    return _spin_site(hilbert, site, [[0.0, 1.0], [1.0, 0.0]])


def _sigmaz(hilbert, site, dtype=None):
    """Pauli Z on ``site``, +1 on the up state (``netket/operator/spin.py:136-166``)."""
    return _spin_site(hilbert, site, [[1.0, 0.0], [0.0, -1.0]])


def _sigmap(hilbert, site, dtype=None):
    """sigma+ = (X + iY) / 2: down -> up (``netket/operator/spin.py:203-233``)."""
    return _spin_site(hilbert, site, [[0.0, 1.0], [0.0, 0.0]])


def _sigmam(hilbert, site, dtype=None):
    """sigma- = (X - iY) / 2: up -> down (``netket/operator/spin.py:169-200``)."""
    return _spin_site(hilbert, site, [[0.0, 0.0], [1.0, 0.0]])


def _sigmay(hilbert, site, dtype=None):
    raise TypeError("sigmay has imaginary matrix elements, not supported on this path; "
                    "sigmay(i) @ sigmay(j) = -(sigmap(i) - sigmam(i)) @ (sigmap(j) - sigmam(j))")


spin = types.SimpleNamespace(identity=_identity, sigmax=_sigmax, sigmay=_sigmay,
                             sigmaz=_sigmaz, sigmap=_sigmap, sigmam=_sigmam)
