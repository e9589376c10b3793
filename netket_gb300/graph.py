"""Graphs and hypercubic lattices with NetKet's edge order (host-side input prep).

Mirrors ``netket.graph`` for the lattices the hot path uses: ``Graph``,
``Grid``/``Hypercube``/``Square``/``Chain`` with ``max_neighbor_order``.

NetKet (``netket/graph/_lattice_edge_logic.py:102-137``) finds neighbour
shells with a KD-tree over the lattice padded by ``order`` cells along periodic
directions, sorts each shell's (padded-index) pairs, maps them to real site
indices and collects them in a Python ``set``; the edges come out in that set's
iteration order.  The order matters: it is the order of LocalOperator terms and
therefore of connected elements.  Here the shells are found with integer
geometry instead (a hypercubic lattice has unit spacing, so shell k is the k-th
smallest squared integer distance realised inside the padded box); the pairs
are generated, sorted and inserted in the same order, so the set iterates
identically.
"""
import itertools

import numpy as np
from scipy.sparse import csr_matrix
from scipy.sparse.csgraph import shortest_path


class Graph:
    """Undirected graph with coloured edges (``netket/graph/graph.py``)."""

    def __init__(self, edges, n_nodes=None):
        edges = list(edges)
        if len(edges) and len(edges[0]) == 3:
            self._edges = [(int(u), int(v)) for u, v, _ in edges]
            self._colors = [int(c) for *_, c in edges]
        elif len(edges) and len(edges[0]) != 2:
            raise ValueError("Edges must be tuple of length 2 (or 3 for colored edges).")
        else:
            self._edges = [(int(u), int(v)) for u, v in edges]
            self._colors = [0] * len(edges)
        if n_nodes is None:
            n_nodes = max(max(e) for e in self._edges) + 1 if self._edges else 0
        self._n = int(n_nodes)

    @property
    def n_nodes(self):
        return self._n

    @property
    def n_edges(self):
        return len(self._edges)

    def nodes(self):
        return range(self._n)

    def edges(self, *, return_color=False, filter_color=None):
        items = list(zip(self._edges, self._colors))
        if filter_color is not None:
            items = [it for it in items if it[1] == filter_color]
        if return_color:
            return [(u, v, c) for (u, v), c in items]
        return [e for e, _ in items]

    @property
    def edge_colors(self):
        return list(self._colors)

    def _csr(self):
        if not self._edges:
            return csr_matrix((self._n, self._n))
        e = np.asarray(self._edges)
        data = np.ones(2 * len(e))
        rows = np.concatenate([e[:, 0], e[:, 1]])
        cols = np.concatenate([e[:, 1], e[:, 0]])
        return csr_matrix((data, (rows, cols)), shape=(self._n, self._n))

    def distances(self):
        """Hop distances between all pairs (``inf`` when disconnected)."""
        return shortest_path(self._csr(), unweighted=True, directed=False)

    def is_bipartite(self):
        adj = self._csr()
        color = np.full(self._n, -1)
        for s in range(self._n):
            if color[s] >= 0:
                continue
            color[s] = 0
            frontier = [s]
            while frontier:
                nxt = []
                for u in frontier:
                    for w in adj.indices[adj.indptr[u]:adj.indptr[u + 1]]:
                        if color[w] < 0:
                            color[w] = 1 - color[u]
                            nxt.append(w)
                        elif color[w] == color[u]:
                            return False
                frontier = nxt
        return True

    def __repr__(self):
        return f"Graph(n_nodes={self._n}, n_edges={len(self._edges)})"


def _hypercubic_edges(extent, pbc, order):
    extent = np.asarray(extent, dtype=np.int64)
    D = len(extent)
    pbc = np.broadcast_to(np.asarray(pbc, dtype=bool), (D,))
    pad = np.where(pbc, order, 0)
    psize = extent + 2 * pad
    # padded sites in C order (the order of np.mgrid over the padded box)
    coords = np.stack(np.meshgrid(*[np.arange(-p, L + p) for p, L in zip(pad, extent)],
                                  indexing="ij"), axis=-1).reshape(-1, D)
    pstride = np.cumprod(np.concatenate([[1], psize[::-1][:-1]]))[::-1]
    rstride = np.cumprod(np.concatenate([[1], extent[::-1][:-1]]))[::-1]
    real_id = (coords % extent) @ rstride
    cutoff2 = (order + 1e-5) ** 2
    rng = int(np.floor(order + 1e-5))
    offsets = [np.array(d) for d in itertools.product(range(-rng, rng + 1), repeat=D)
               if 0 < sum(x * x for x in d) <= cutoff2 and all(abs(x) < s for x, s in zip(d, psize))]
    shells = sorted({int(d @ d) for d in offsets})[:order]
    out = []
    for k, v in enumerate(shells):
        pairs = []
        for d in offsets:
            if int(d @ d) != v:
                continue
            nb = coords + d
            ok = np.all((nb >= -pad) & (nb < extent + pad), axis=1)
            a = ((coords[ok] + pad) @ pstride)
            b = ((nb[ok] + pad) @ pstride)
            keep = a < b
            pairs.append(np.stack([a[keep], b[keep]], axis=1))
        pairs = np.concatenate(pairs) if pairs else np.zeros((0, 2), dtype=np.int64)
        pairs = pairs[np.lexsort((pairs[:, 1], pairs[:, 0]))]
        uniq = set()
        for pa, pb in pairs:
            u = int(real_id[pa])
            w = int(real_id[pb])
            if u == w:
                raise RuntimeError(f"Lattice contains self-referential edge {(u, w)} of order {k}")
            if u > w:
                u, w = w, u
            uniq.add((u, w))
        out.extend((u, w, k) for (u, w) in uniq)
    return out


class Lattice(Graph):
    """Hypercubic lattice with unit basis vectors and one site per cell."""

    def __init__(self, extent, pbc=True, max_neighbor_order=None):
        self.extent = np.asarray(extent, dtype=int)
        self.pbc = np.broadcast_to(np.asarray(pbc, dtype=bool), (len(self.extent),)).copy()
        self.max_neighbor_order = 1 if max_neighbor_order is None else int(max_neighbor_order)
        edges = _hypercubic_edges(self.extent, self.pbc, self.max_neighbor_order)
        super().__init__(edges, int(np.prod(self.extent)))

    @property
    def ndim(self):
        return len(self.extent)

    def __repr__(self):
        return (f"Lattice(extent={self.extent.tolist()}, pbc={self.pbc.tolist()}, "
                f"max_neighbor_order={self.max_neighbor_order})")


def Grid(extent, *, pbc=True, max_neighbor_order=None):
    return Lattice(extent, pbc, max_neighbor_order)


def Hypercube(length, n_dim=1, *, pbc=True, max_neighbor_order=None):
    if not isinstance(length, int) or length <= 0:
        raise TypeError("Argument `length` must be a positive integer")
    return Lattice([length] * n_dim, pbc, max_neighbor_order)


def Square(length, *, pbc=True, max_neighbor_order=None):
    return Hypercube(length, 2, pbc=pbc, max_neighbor_order=max_neighbor_order)


def Chain(length, *, pbc=True, max_neighbor_order=None):
    return Hypercube(length, 1, pbc=pbc, max_neighbor_order=max_neighbor_order)
