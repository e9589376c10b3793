"""Shared helpers for the GPU parity tests (oracle builders for the same
Hamiltonians and parameters the product uses)."""
import numpy as np

from oracle import graph as og
from oracle import operator as oop
from oracle import rbm as orbm


def oracle_graph(g):
    return og.Graph(g.edges(return_color=True), g.n_nodes)


def oracle_params(vs_or_flat, N, M):
    flat = vs_or_flat if isinstance(vs_or_flat, np.ndarray) else vs_or_flat.cpu().numpy()
    return orbm.unravel(flat.astype(np.float64), N, M)


def oracle_heisenberg(g, J=1.0, sign_rule=None):
    return oop.heisenberg(g.n_nodes, oracle_graph(g), J, sign_rule)


def oracle_local(op):
    """Oracle LocalOperator with the same terms as a product LocalOperator."""
    return oop.LocalOperator(op.hilbert.size, op.operators, op.acting_on, constant=op.constant,
                             mel_cutoff=op.mel_cutoff)
