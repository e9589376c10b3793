"""Graphs and lattices with NetKet's edge order (host-side input prep).

Mirrors ``netket.graph``: ``Graph``, ``Lattice`` (basis vectors, site offsets,
``max_neighbor_order``), ``Grid`` / ``Hypercube`` / ``Cube`` / ``Square`` /
``Chain`` and the hexagonal ``Triangular`` / ``Honeycomb`` / ``Kagome``.

NetKet (``netket/graph/_lattice_edge_logic.py:102-137``) finds neighbour
shells with a KD-tree over the lattice padded by ``order`` cells along periodic
directions, sorts each shell's (padded-index) pairs, maps them to real site
indices and collects them in a Python ``set``; the edges come out in that set's
iteration order.  The order matters: it is the order of LocalOperator terms and
therefore of connected elements.  Here the shells are found with integer
geometry instead (a hypercubic lattice has unit spacing, so shell k is the k-th
smallest squared integer distance realised inside the padded box); the pairs
are generated, sorted and inserted in the same order, so the set iterates
identically.  Lattices with other basis vectors or several sites per cell
use the same shell rule on real-space distances (pairs within
``order * max|basis vector| + distance_atol`` of each other, grouped into
shells of equal length, the first ``order`` shells kept).
"""
import itertools
import warnings

import numpy as np
from scipy.sparse import csr_matrix
from scipy.sparse.csgraph import shortest_path
from scipy.spatial import cKDTree


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


def _cell_sites(basis, extent, offsets, pad):
    """Sites of the box of cells [-pad, extent + pad) in C order, sublattice
    fastest: (real-space positions, real site index of each)."""
    D, S = len(extent), len(offsets)
    cells = np.stack(np.meshgrid(*[np.arange(-p, L + p) for p, L in zip(pad, extent)],
                                 indexing="ij"), axis=-1).reshape(-1, D)
    pos = (cells @ basis)[:, None, :] + offsets[None, :, :]
    radix = np.cumprod(np.concatenate([[S], extent[::-1][:-1]]))[::-1]
    ids = ((cells % extent) @ radix)[:, None] + np.arange(S)[None, :]
    return pos.reshape(-1, D), ids.reshape(-1)


def _shell_edges(positions, ids, cutoff, order):
    """Edges of the first ``order`` distance shells among pairs within
    ``cutoff``: per shell the (i < j) pairs of padded sites in lexicographic
    order, mapped to real sites (smaller first) and collected in a set."""
    pairs = cKDTree(positions).query_pairs(cutoff, output_type="ndarray")
    if len(pairs) == 0:
        return []
    pairs = np.sort(pairs, axis=1)
    d = np.linalg.norm(positions[pairs[:, 0]] - positions[pairs[:, 1]], axis=1)
    # shells: distances equal up to rounding, clustered along the sorted lengths
    srt = np.sort(d)
    breaks = srt[1:][np.diff(srt) > 1e-7]
    edges_of_shell = np.concatenate([[srt[0]], breaks])
    shell = np.searchsorted(edges_of_shell, d, side="right") - 1
    out = []
    for k in range(order):
        pk = pairs[shell == k]
        pk = pk[np.lexsort((pk[:, 1], pk[:, 0]))]
        uniq = set()
        for a, b in pk:
            u, w = int(ids[a]), int(ids[b])
            if u == w:
                raise RuntimeError(f"Lattice contains self-referential edge {(u, w)} of order {k}")
            uniq.add((u, w) if u < w else (w, u))
        out.extend((u, w, k) for (u, w) in uniq)
    return out


def _lattice_edges(basis, extent, offsets, pbc, order, distance_atol=1e-5):
    pad = np.where(pbc, order, 0)
    pos, ids = _cell_sites(basis, extent, offsets, pad)
    cutoff = order * np.linalg.norm(basis, axis=1).max() + distance_atol
    return _shell_edges(pos, ids, cutoff, order)


class Lattice(Graph):
    """A lattice of ``extent`` unit cells spanned by the rows of
    ``basis_vectors``, with the sites of ``site_offsets`` in every cell
    (``netket/graph/lattice.py:166-330``); site index = cell index in C order
    times the sites per cell plus the sublattice.  Edges join the first
    ``max_neighbor_order`` neighbour shells, coloured by shell."""

    def __init__(self, basis_vectors, extent, *, pbc=True, site_offsets=None,
                 distance_atol=1e-5, max_neighbor_order=None):
        basis = np.atleast_2d(np.asarray(basis_vectors, dtype=np.float64))
        if basis.ndim != 2 or basis.shape[0] != basis.shape[1]:
            raise ValueError("basis_vectors must be a square (ndim, ndim) matrix")
        D = basis.shape[0]
        self.basis_vectors = basis
        self.extent = np.asarray(extent, dtype=int)
        if self.extent.shape != (D,):
            raise ValueError(f"extent must have {D} entries")
        if isinstance(pbc, (bool, np.bool_)):
            pbc = [bool(pbc)] * D
        if len(pbc) != D or not all(isinstance(b, (bool, np.bool_)) for b in pbc):
            raise ValueError("pbc must be either a boolean or a list of booleans with the "
                             "same dimension as the lattice")
        self.pbc = np.asarray(pbc, dtype=bool)
        self.site_offsets = (np.zeros((1, D)) if site_offsets is None
                             else np.atleast_2d(np.asarray(site_offsets, dtype=np.float64)))
        self.max_neighbor_order = 1 if max_neighbor_order is None else int(max_neighbor_order)
        hypercubic = (np.array_equal(basis, np.eye(D)) and len(self.site_offsets) == 1
                      and not np.any(self.site_offsets))
        if hypercubic:
            edges = _hypercubic_edges(self.extent, self.pbc, self.max_neighbor_order)
        else:
            edges = _lattice_edges(basis, self.extent, self.site_offsets, self.pbc,
                                   self.max_neighbor_order, distance_atol)
        super().__init__(edges, int(np.prod(self.extent)) * len(self.site_offsets))

    @property
    def ndim(self):
        return len(self.extent)

    @property
    def positions(self):
        pos, _ = _cell_sites(self.basis_vectors, self.extent, self.site_offsets,
                             np.zeros(self.ndim, dtype=int))
        return pos

    def __repr__(self):
        return (f"Lattice(extent={self.extent.tolist()}, pbc={self.pbc.tolist()}, "
                f"n_sites_per_cell={len(self.site_offsets)}, "
                f"max_neighbor_order={self.max_neighbor_order})")


def Grid(extent, *, pbc=True, max_neighbor_order=None):
    extent = list(extent)
    return Lattice(np.eye(len(extent)), extent, pbc=pbc, max_neighbor_order=max_neighbor_order)


def Hypercube(length, n_dim=1, *, pbc=True, max_neighbor_order=None):
    if not isinstance(length, int) or length <= 0:
        raise TypeError("Argument `length` must be a positive integer")
    return Grid([length] * n_dim, pbc=pbc, max_neighbor_order=max_neighbor_order)


def Cube(length, *, pbc=True, max_neighbor_order=None):
    return Hypercube(length, 3, pbc=pbc, max_neighbor_order=max_neighbor_order)


_HEX_BASIS = [[1.0, 0.0], [0.5, 0.75 ** 0.5]]


def _hexagonal(extent, site_offsets, pbc, max_neighbor_order):
    """``netket/graph/common_lattices.py:435-455``: basis (1, 0), (1/2, sqrt(3)/2);
    a periodic direction of at most 2 cells only warns, as there."""
    extent = list(extent)
    pbcs = [pbc] * 2 if isinstance(pbc, bool) else list(pbc)
    for i in range(2):
        if extent[i] <= 2 and pbcs[i]:
            warnings.warn(f"Lattice with periodic boundary conditions along direction {i} "
                          f"has only {extent[i]} cells: neighbours may be repeated",
                          UserWarning, stacklevel=3)
    return Lattice(_HEX_BASIS, extent, pbc=pbc, site_offsets=site_offsets,
                   max_neighbor_order=max_neighbor_order)


def Triangular(extent, *, pbc=True, max_neighbor_order=None):
    return _hexagonal(extent, None, pbc, max_neighbor_order)


def Honeycomb(extent, *, pbc=True, max_neighbor_order=None):
    """Two sites per cell (``common_lattices.py:504-538``)."""
    return _hexagonal(extent, [[0.5, 0.5 / 3 ** 0.5], [1.0, 1.0 / 3 ** 0.5]], pbc,
                      max_neighbor_order)


def Kagome(extent, *, pbc=True, max_neighbor_order=None):
    """Three sites per cell (``common_lattices.py:540-574``)."""
    return _hexagonal(extent, [[0.5, 0.0], [0.25, 0.75 ** 0.5 / 2], [0.75, 0.75 ** 0.5 / 2]],
                      pbc, max_neighbor_order)


def Square(length, *, pbc=True, max_neighbor_order=None):
    return Hypercube(length, 2, pbc=pbc, max_neighbor_order=max_neighbor_order)


def Chain(length, *, pbc=True, max_neighbor_order=None):
    return Hypercube(length, 1, pbc=pbc, max_neighbor_order=max_neighbor_order)
