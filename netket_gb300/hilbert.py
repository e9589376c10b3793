"""Spin-1/2 Hilbert space (``netket.hilbert.Spin`` for s = 1/2).

States are int8 tensors with values +1 / -1 (NetKet's new ordering,
``netket/hilbert/spin.py:167-172``); local index 0 <-> +1, 1 <-> -1.
Random states come from the CUDA kernel ``vmck_random_states``.
"""
import numpy as np
import torch

from . import _native as nat


class Spin:
    """``netket.hilbert.Spin`` for s = 1/2 (``netket/hilbert/spin.py:110-207``):
    ``total_sz`` fixes the number of down spins; the basis ordering is the
    reference's default (``inverted_ordering=False``: +1 = up); unconstrained
    spaces multiply (``Spin(0.5) ** 8``, ``a * b``) into longer chains."""

    def __init__(self, s=0.5, N=1, total_sz=None, *, constraint=None, inverted_ordering=False):
        if s != 0.5:
            raise NotImplementedError("only spin-1/2 is supported")
        if constraint is not None:
            raise NotImplementedError("Spin: custom constraints are not supported (total_sz is)")
        if inverted_ordering:
            raise NotImplementedError("Spin: inverted_ordering=True (-1 = up) is not supported; "
                                      "the kernels use the default +1 = up ordering")
        if int(N) < 1:
            raise ValueError(f"Spin: N must be positive, got {N}")
        self.s = 0.5
        self.N = int(N)
        if total_sz is not None:
            two_sz = round(2 * total_sz)
            if (self.N + two_sz) % 2 != 0 or abs(two_sz) > self.N:
                raise ValueError(f"total_sz={total_sz} is incompatible with N={self.N}")
        self.total_sz = total_sz

    @property
    def size(self):
        return self.N

    @property
    def local_size(self):
        return 2

    @property
    def local_states(self):
        return [1, -1]

    @property
    def shape(self):
        return (2,) * self.N

    @property
    def constrained(self):
        return self.total_sz is not None

    @property
    def n_down(self):
        """Number of down spins fixed by ``total_sz`` (None if unconstrained)."""
        if self.total_sz is None:
            return None
        return (self.N - round(2 * self.total_sz)) // 2

    def random_state(self, seed, size, stream_id=0):
        """(size, N) int8 device tensor: uniform, or a uniformly random
        arrangement of the fixed number of down spins."""
        out = torch.empty((int(size), self.N), dtype=torch.int8, device=nat.device())
        nd = -1 if self.n_down is None else self.n_down
        nat.check(nat.lib().vmck_random_states(nat.stream(), nat.ptr(out), int(size), self.N, nd,
                                               int(seed) & (2**64 - 1), int(stream_id)))
        return out

    @staticmethod
    def states_to_local_indices(x):
        return ((1 - x.to(torch.int16)) // 2).to(torch.int8)

    @staticmethod
    def local_indices_to_states(i):
        return (1 - 2 * i.to(torch.int16)).to(torch.int8)

    @property
    def n_states(self):
        if self.total_sz is None:
            return 2**self.N
        from math import comb
        return comb(self.N, self.n_down)

    def all_states(self):
        """Every basis state (device int8), first site most significant."""
        return torch.from_numpy(1 - 2 * self._all_local_indices()).to(nat.device())

    def _all_local_indices(self):
        """(n_states, N) int8 local indices of every basis state, in order."""
        if self.N > 26:
            raise ValueError("Hilbert space too large to enumerate")
        code = np.arange(2 ** self.N, dtype=np.int64)
        if self.n_down is not None:
            pop = np.zeros_like(code)
            for k in range(self.N):
                pop += (code >> k) & 1
            code = code[pop == self.n_down]
        shifts = np.arange(self.N - 1, -1, -1, dtype=np.int64)
        return ((code[:, None] >> shifts) & 1).astype(np.int8)

    def __mul__(self, other):
        """Spin x Spin: one longer unconstrained chain (``spin.py:201-207``)."""
        if not isinstance(other, Spin):
            return NotImplemented
        if self.constrained or other.constrained:
            raise NotImplementedError("products of constrained Spin spaces are not supported")
        return Spin(0.5, self.N + other.N)

    def __pow__(self, n):
        if not isinstance(n, int) or n < 1:
            return NotImplemented
        if self.constrained:
            raise NotImplementedError("powers of a constrained Spin space are not supported")
        return Spin(0.5, self.N * n)

    def __eq__(self, other):
        return isinstance(other, Spin) and (self.N, self.total_sz) == (other.N, other.total_sz)

    def __hash__(self):
        return hash((self.N, self.total_sz))

    def __repr__(self):
        tsz = "" if self.total_sz is None else f", total_sz={self.total_sz}"
        return f"Spin(s=1/2{tsz}, N={self.N})"
