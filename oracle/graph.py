"""Oracle: lattice edges in NetKet's order (test infrastructure only).

Restates ``netket/graph/_lattice_edge_logic.py:26-137`` (site positions, padded
shells for periodic boundaries, KD-tree neighbour search, shell binning by
``netket/utils/float.py:22-47`` ``comparable``) and ``Graph.edges`` /
``distances`` / ``is_bipartite`` (``netket/graph/graph.py:135-180``).

The order of edges matters: it fixes the order of LocalOperator terms and
therefore of connected elements.  NetKet collects each neighbour shell into a
Python ``set`` of ``(i, j)`` tuples and emits them in set-iteration order; this
module builds the same set with the same insertion order, so the iteration
order is identical.
"""
from collections import deque

import numpy as np
from scipy.sparse import find, triu
from scipy.spatial import cKDTree


def comparable(x, bin_density=3326400, offset=5413 / 15629):
    # netket/utils/float.py:22-47
    return np.asarray(np.rint(np.asarray(x) * bin_density + offset), dtype=int)


def _site_positions(basis, extent, offsets, extra):
    # netket/graph/_lattice_edge_logic.py:26-48
    lo = -extra
    hi = extent + extra
    ranges = [slice(a, b) for a, b in zip(lo, hi)] + [slice(0, len(offsets))]
    coords = np.mgrid[ranges].reshape(len(extent) + 1, -1).T
    pos = coords[:, :-1] @ basis
    pos = pos.reshape(-1, len(offsets), len(extent)) + offsets
    return coords, pos.reshape(-1, len(extent))


def _site_index(coords, extent, n_offsets):
    # netket/graph/_lattice_edge_logic.py:51-68
    cell, sl = coords[:, :-1] % extent, coords[:, -1]
    radix = np.cumprod([n_offsets, *extent[:0:-1]])[::-1]
    return cell @ radix + sl


def lattice_edges(extent, pbc=True, max_neighbor_order=1, distance_atol=1e-5):
    """Colored edges ``[(i, j, color), ...]`` of a hypercubic lattice.

    Follows ``get_nn_edges`` (``_lattice_edge_logic.py:102-137``) with unit basis
    vectors and one site per cell (the Hypercube/Square/Chain constructors,
    ``netket/graph/common_lattices.py:143-230``).
    """
    extent = np.asarray(extent, dtype=int)
    ndim = len(extent)
    basis = np.eye(ndim)
    offsets = np.zeros((1, ndim))
    pbc = np.broadcast_to(np.asarray(pbc, dtype=bool), (ndim,))
    order = int(max_neighbor_order)
    extra = np.where(pbc, order, 0)
    coords, pos = _site_positions(basis, extent, offsets, extra)
    ids = _site_index(coords, extent, len(offsets))
    cutoff = order * np.linalg.norm(basis, axis=1).max() + distance_atol
    tree = cKDTree(pos)
    dmat = tree.sparse_distance_matrix(tree, cutoff)
    row, col, dst = find(triu(dmat))
    _, ii = np.unique(comparable(dst), return_inverse=True)
    shells = [sorted(zip(row[ii == k], col[ii == k])) for k in range(order)]
    out = []
    for k, shell in enumerate(shells):
        uniq = set()
        for a, b in shell:
            a, b = ids[a], ids[b]
            if a == b:
                raise RuntimeError(f"self-referential edge {(a, b)} of order {k}")
            if a > b:
                a, b = b, a
            uniq.add((a, b))
        for e in uniq:
            out.append((int(e[0]), int(e[1]), k))
    return out


class Graph:
    """Undirected colored graph with NetKet's edge accessors."""

    def __init__(self, edges, n_nodes=None):
        edges = list(edges)
        if len(edges) and len(edges[0]) == 3:
            self._edges = [(int(u), int(v)) for u, v, _ in edges]
            self._colors = [int(c) for *_, c in edges]
        else:
            self._edges = [(int(u), int(v)) for u, v in edges]
            self._colors = [0] * len(edges)
        if n_nodes is None:
            n_nodes = max(max(e) for e in self._edges) + 1 if self._edges else 0
        self.n_nodes = int(n_nodes)

    def edges(self, return_color=False, filter_color=None):
        items = list(zip(self._edges, self._colors))
        if filter_color is not None:
            items = [it for it in items if it[1] == filter_color]
        if return_color:
            return [(u, v, c) for (u, v), c in items]
        return [e for e, _ in items]

    @property
    def edge_colors(self):
        return list(self._colors)

    def _adjacency(self):
        adj = [[] for _ in range(self.n_nodes)]
        for u, v in self._edges:
            adj[u].append(v)
            adj[v].append(u)
        return adj

    def distances(self):
        """All-pairs hop distances (igraph ``distances``), ``inf`` if disconnected."""
        adj = self._adjacency()
        d = np.full((self.n_nodes, self.n_nodes), np.inf)
        for s in range(self.n_nodes):
            d[s, s] = 0
            q = deque([s])
            while q:
                u = q.popleft()
                for w in adj[u]:
                    if d[s, w] == np.inf:
                        d[s, w] = d[s, u] + 1
                        q.append(w)
        return d

    def is_bipartite(self):
        adj = self._adjacency()
        col = [-1] * self.n_nodes
        for s in range(self.n_nodes):
            if col[s] >= 0:
                continue
            col[s] = 0
            q = deque([s])
            while q:
                u = q.popleft()
                for w in adj[u]:
                    if col[w] < 0:
                        col[w] = 1 - col[u]
                        q.append(w)
                    elif col[w] == col[u]:
                        return False
        return True


def Hypercube(length, n_dim=1, pbc=True, max_neighbor_order=1):
    n = length**n_dim
    return Graph(lattice_edges([length] * n_dim, pbc, max_neighbor_order), n)


def Square(length, pbc=True, max_neighbor_order=1):
    return Hypercube(length, 2, pbc, max_neighbor_order)


def Chain(length, pbc=True, max_neighbor_order=1):
    return Hypercube(length, 1, pbc, max_neighbor_order)


def compute_clusters(graph, d_max):
    """Exchange clusters: pairs (i<j) with hop distance <= d_max.

    ``netket/sampler/rules/exchange.py:190-205`` (row-major ``argwhere`` order).
    """
    dist = np.asarray(graph.distances())
    cl = np.argwhere(dist <= d_max)
    return cl[cl[:, 0] < cl[:, 1]].astype(np.int64)
