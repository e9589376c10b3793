"""Generate golden vectors by executing NetKet's own source in this container.

NetKet cannot be imported here (jax, flax, numba and igraph are absent), but the
functions that pin the hot path are plain numpy / numba-kernel code.  This
script parses the reference source files, extracts the named functions, strips
their decorators (``numba.jit`` becomes a plain Python function, ``jax.jit`` is
dropped) and executes them with numpy standing in for ``jax.numpy``.  Nothing
from the reference is copied into the repository: only the input/output arrays
are written, to ``tests/golden/*.npz``.

Covered:
  edges.npz      get_nn_edges (graph/_lattice_edge_logic.py:102-137) on several lattices
  ising.npz      IsingNumba._flattened_kernel (operator/_ising/numba.py:101-132)
  localop.npz    pack_internals + LocalOperatorNumba._get_conn_flattened_kernel
                 (operator/_local_operator/compile_helpers.py:29-171,
                 operator/_local_operator/numba.py:132-240) for Heisenberg
                 (operator/_heisenberg.py:33-132 via operator/_graph_operator.py:47-145)
                 and Ising-as-LocalOperator
  logcosh.npz    log_cosh (nn/activation.py:78-84)
  stats.npz      _statistics (stats/mc_stats_old.py:88-196)
  online_stats.npz  OnlineStats update (_src/stats/online_stats/kernels.py:23-190) and
                 read-outs (accumulator.py:240-447) over chunk sequences
  hamiltonian_rule.npz  HamiltonianRuleNumba proposal (sampler/rules/hamiltonian.py:
                 84-127: get_conn_flattened, _choose, n_conn) and IsingJax n_conn
  hamiltonian_rule_pauli.npz  HamiltonianRuleJax.transition (sampler/rules/
                 hamiltonian.py:166-213) over the reference's PauliStrings kernel
  spring.npz     the same updates with SPRING momentum / proj_reg
  ngd.npz        _prepare_input + _compute_srt_update + _compute_sr_update
                 (_src/ngd/sr_srt_common.py:45-101, _src/ngd/srt.py:22-96,
                 _src/ngd/sr.py:23-80) with cholesky / pinv_smooth /
                 cholesky_with_fallback (optimizer/solver/solvers.py,
                 _src/solvers/nan_fallback.py:22-45)

Run:  python tests/golden/make_golden.py REFERENCE_ROOT   (or set NETKET_REFERENCE_ROOT)
"""
import __future__
import ast
import os
import sys
import types

import numpy as np
import scipy.linalg
import scipy.sparse
from scipy.sparse import find, triu
from scipy.spatial import cKDTree

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

# The reference checkout to read: the first argument or $NETKET_REFERENCE_ROOT
# (required; the fixtures are generated from that tree's own source files).
REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("NETKET_REFERENCE_ROOT")
if not REF:
    sys.exit("usage: make_golden.py REFERENCE_ROOT (or set NETKET_REFERENCE_ROOT): the path of "
             "the NetKet source tree whose functions generate the fixtures")
NK = os.path.join(REF, "netket")


def load(relpath, names, ns, class_name=None):
    """Exec the named top-level (or class-level) functions of a reference file."""
    path = os.path.join(NK, relpath)
    tree = ast.parse(open(path).read(), filename=path)
    body = tree.body
    if class_name is not None:
        body = next(n for n in tree.body if isinstance(n, ast.ClassDef)
                    and n.name == class_name).body
    nodes = [n for n in body if isinstance(n, ast.FunctionDef) and n.name in names]
    missing = set(names) - {n.name for n in nodes}
    if missing:
        raise RuntimeError(f"{relpath}: functions not found: {missing}")
    for n in nodes:
        n.decorator_list = []
    mod = ast.Module(body=nodes, type_ignores=[])
    code = compile(mod, path, "exec", flags=__future__.annotations.compiler_flag,
                   dont_inherit=True)
    exec(code, ns)
    return ns


# ---------------------------------------------------------------- shims
numba_stub = types.SimpleNamespace(jit=lambda *a, **k: (lambda f: f))


def lax_cond(pred, true_fun, false_fun, *operands):
    return true_fun(*operands) if bool(pred) else false_fun(*operands)


jax_stub = types.SimpleNamespace(
    lax=types.SimpleNamespace(cond=lax_cond, add=np.add,
                              collapse=lambda x, a, b: x.reshape((-1,) + x.shape[b:])),
    Array=np.ndarray,
)


class FakeHilbert:
    def __init__(self, N):
        self.size = N
        self.shape = [2] * N

    def size_at_index(self, i):
        return 2


def ravel_identity(x):
    x = np.asarray(x)
    return x, (lambda y: y)


# ---------------------------------------------------------------- edges
def gen_edges():
    ns = {"np": np, "cKDTree": cKDTree, "find": find, "triu": triu}
    load("utils/float.py", ["comparable"], ns)
    load("graph/_lattice_edge_logic.py",
         ["create_site_positions", "site_to_idx", "create_padded_sites",
          "get_naive_edges", "get_nn_edges"], ns)
    cases = {
        "chain16": ([16], True, 1), "chain5": ([5], True, 1), "chain8_obc": ([8], False, 1),
        "chain14_nnn": ([14], True, 2), "square4": ([4, 4], True, 1),
        "square6_nnn": ([6, 6], True, 2), "square10_nnn": ([10, 10], True, 2),
        "square16": ([16, 16], True, 1), "cube3": ([3, 3, 3], True, 1),
    }
    out = {}
    for name, (extent, pbc, order) in cases.items():
        d = len(extent)
        e = ns["get_nn_edges"](np.eye(d), np.asarray(extent), np.zeros((1, d)),
                               np.array([pbc] * d), 1e-5, order)
        out[name] = np.array(e, dtype=np.int64).reshape(-1, 3)
        out[name + "__meta"] = np.array(extent + [int(pbc), order], dtype=np.int64)
    np.savez_compressed(os.path.join(HERE, "edges.npz"), **out)
    return out


def gen_lattice_edges():
    """get_nn_edges (graph/_lattice_edge_logic.py:102-137) and the site
    positions (create_site_positions, :26-48) for lattices with non-unit basis
    vectors and several sites per cell, plus hypercubic cases run through the
    same general code path."""
    ns = {"np": np, "cKDTree": cKDTree, "find": find, "triu": triu}
    load("utils/float.py", ["comparable"], ns)
    load("graph/_lattice_edge_logic.py",
         ["create_site_positions", "site_to_idx", "create_padded_sites",
          "get_naive_edges", "get_nn_edges"], ns)
    hexb = [[1.0, 0.0], [0.5, 0.75 ** 0.5]]
    honey = [[0.5, 0.5 / 3 ** 0.5], [1.0, 1.0 / 3 ** 0.5]]
    kag = [[0.5, 0.0], [0.25, 0.75 ** 0.5 / 2], [0.75, 0.75 ** 0.5 / 2]]
    cases = {
        "triangular3": (hexb, [3, 3], None, [True, True], 1),
        "triangular4x3_nnn": (hexb, [4, 3], None, [True, True], 2),
        "triangular4_obc": (hexb, [4, 4], None, [False, False], 2),
        "triangular5x4_mixed": (hexb, [5, 4], None, [True, False], 3),
        "honeycomb3": (hexb, [3, 3], honey, [True, True], 1),
        "honeycomb4_3rd": (hexb, [4, 4], honey, [True, True], 3),
        "honeycomb3x4_obc": (hexb, [3, 4], honey, [False, True], 2),
        "kagome3": (hexb, [3, 3], kag, [True, True], 1),
        "kagome4_nnn": (hexb, [4, 4], kag, [True, True], 2),
        "rect_two_site": ([[1.0, 0.0], [0.0, 1.5]], [4, 3], [[0.0, 0.0], [0.5, 0.75]],
                          [True, True], 3),
        "square5_via_general": ([[1.0, 0.0], [0.0, 1.0]], [5, 5], None, [True, True], 2),
    }
    out = {}
    for name, (basis, extent, offsets, pbc, order) in cases.items():
        basis = np.asarray(basis)
        d = basis.shape[0]
        offs = np.zeros((1, d)) if offsets is None else np.asarray(offsets)
        e = ns["get_nn_edges"](basis, np.asarray(extent), offs, np.array(pbc), 1e-5, order)
        _, pos = ns["create_site_positions"](basis, np.asarray(extent), offs)
        out[name + "__edges"] = np.array(e, dtype=np.int64).reshape(-1, 3)
        out[name + "__basis"] = basis
        out[name + "__extent"] = np.array(extent, dtype=np.int64)
        out[name + "__offsets"] = offs
        out[name + "__pbc"] = np.array(pbc)
        out[name + "__order"] = np.array(order)
        out[name + "__positions"] = pos
    np.savez_compressed(os.path.join(HERE, "lattice_edges.npz"), **out)


# ---------------------------------------------------------------- operators
def gen_ising(edges):
    ns = {"np": np}
    load("operator/_ising/numba.py", ["_flattened_kernel"], ns, class_name="IsingNumba")
    rng = np.random.default_rng(1234)
    out = {}
    for name, N, h, J in [("chain16", 16, 1.0, 1.0), ("chain5", 5, 0.7, -1.3),
                          ("square4", 16, 0.5, 1.0)]:
        e = edges[name][:, :2]
        x_ids = rng.integers(0, 2, size=(37, N)).astype(np.int8)
        sections = np.zeros(x_ids.shape[0], dtype=np.int64)
        xp_ids, mels = ns["_flattened_kernel"](x_ids, sections, e.astype(np.intp),
                                               np.float64(h), np.float64(J))
        out[name + "__x_ids"] = x_ids
        out[name + "__xp_ids"] = xp_ids
        out[name + "__mels"] = mels
        out[name + "__hJ"] = np.array([h, J])
    np.savez_compressed(os.path.join(HERE, "ising.npz"), **out)


def gen_localop(edges):
    from oracle import graph as og, operator as oop
    ns = {"np": np, "numba": numba_stub, "sparse": scipy.sparse}
    load("operator/_local_operator/compile_helpers.py",
         ["pack_internals", "_append_matrix", "_append_matrix_sparse",
          "_number_to_state", "max_nonzero_per_row"], ns)
    load("operator/_local_operator/numba.py", ["_get_conn_flattened_kernel"], ns,
         class_name="LocalOperatorNumba")
    # GraphOperator / Heisenberg term construction, recorded through a fake class
    rec = {}

    def recorder(hilbert, operators, acting_on, dtype=None):
        rec["ops"], rec["aon"] = operators, acting_on
        return rec

    gns = {"np": np, "Sequence": (list, tuple), "Graph": None, "_LocalOperator": recorder}
    load("operator/_graph_operator.py", ["check_acting_on_subspace", "GraphOperator"], gns)
    load("operator/_heisenberg.py", ["Heisenberg"], gns)

    rng = np.random.default_rng(4321)
    out = {}
    cases = [
        ("heis_chain16", "chain16", 1.0, None), ("heis_square4", "square4", 1.0, None),
        ("heis_square4_nosign", "square4", 1.0, False),
        ("j1j2_square6", "square6_nnn", [1.0, 0.5], None),
        ("j1j2_chain14", "chain14_nnn", [1.0, 0.2], None),
        ("j1j2_square10", "square10_nnn", [1.0, 0.5], None),
    ]
    for name, gname, J, sr in cases:
        e = edges[gname]
        meta = edges[gname + "__meta"]
        N = int(np.prod(meta[:-2]))
        g = og.Graph([tuple(r) for r in e], N)
        kwargs = {"cls": recorder}
        if sr is not None:
            kwargs["sign_rule"] = sr
        gns["Heisenberg"](FakeHilbert(N), g, J, **kwargs)
        ops = [np.asarray(o, dtype=np.float64) for o in rec["ops"]]
        aon = [tuple(int(s) for s in a) for a in rec["aon"]]
        _store_localop(ns, out, name, N, ops, aon, rng, oop)
    # Ising as a LocalOperator: 1-site and 2-site groups
    e = edges["chain5"][:, :2]
    ops = [-0.7 * oop.SIGMAX for _ in range(5)] + [1.3 * np.kron(oop.SIGMAZ, oop.SIGMAZ)
                                                   for _ in e]
    aon = [(i,) for i in range(5)] + [tuple(int(s) for s in r) for r in e]
    _store_localop(ns, out, "ising_local_chain5", 5, ops, aon, rng, oop)
    np.savez_compressed(os.path.join(HERE, "localop.npz"), **out)


def _store_localop(ns, out, name, N, ops, aon, rng, oop):
    # _operators_dict summation (base.py:135-147); acting_on are sorted already
    d = {}
    for o, a in zip(ops, aon):
        assert list(a) == sorted(a)
        d[a] = d[a] + o if a in d else o
    packed = ns["pack_internals"](FakeHilbert(N), d, np.float64(0.0), np.float64, 1e-10)
    n = 23
    x_ids = rng.integers(0, 2, size=(n, N)).astype(np.int8)
    sections = np.zeros(n, dtype=np.int64)
    xp_ids, mels = ns["_get_conn_flattened_kernel"](
        x_ids, sections, packed["basis"], np.array(0.0), packed["diag_mels"],
        packed["n_conns"], packed["mels"], packed["x_prime"], packed["acting_on"],
        packed["acting_size"], packed["nonzero_diagonal"], False)
    out[name + "__N"] = np.array(N)
    out[name + "__aon"] = np.array([list(a) + [-1] * (2 - len(a)) for a in d.keys()])
    out[name + "__ops"] = np.array([np.pad(m, ((0, 4 - m.shape[0]), (0, 4 - m.shape[1])))
                                    for m in d.values()])
    out[name + "__sizes"] = np.array([len(a) for a in d.keys()])
    out[name + "__x_ids"] = x_ids
    out[name + "__xp_ids"] = xp_ids
    out[name + "__mels"] = mels
    out[name + "__sections"] = sections
    out[name + "__max_conn_numba"] = np.array(packed["max_conn_size"])
    # max_conn_size of the JAX packer (compile_helpers.py:174-218), via the same helper
    sizes = np.array([len(a) for a in d.keys()])
    K, nz = 0, False
    for s in np.unique(sizes):
        sub = {a: m for a, m in d.items() if len(a) == s}
        p = ns["pack_internals"](FakeHilbert(N), sub, 0, np.float64, 1e-10)
        k = int(p["max_conn_size"]) - (1 if p["nonzero_diagonal"] else 0)
        K += k
        nz = nz or bool(p["nonzero_diagonal"])
    out[name + "__max_conn_jax"] = np.array(K + (1 if nz else 0))


# ---------------------------------------------------------------- Hamiltonian rule
def gen_hamiltonian_rule(edges):
    """HamiltonianRuleNumba.transition (sampler/rules/hamiltonian.py:84-127):
    get_conn_flattened, _choose with given uniforms, n_conn of the proposals
    (_discrete_operator.py:173-200); and IsingJax's n_conn (_ising/jax.py:168-175)."""
    from oracle import operator as oop
    import math
    ns = {"np": np, "numba": numba_stub, "sparse": scipy.sparse, "math": math}
    load("operator/_local_operator/compile_helpers.py",
         ["pack_internals", "_append_matrix", "_append_matrix_sparse",
          "_number_to_state", "max_nonzero_per_row"], ns)
    load("operator/_local_operator/numba.py", ["_get_conn_flattened_kernel"], ns,
         class_name="LocalOperatorNumba")
    load("sampler/rules/hamiltonian.py", ["_choose"], ns)
    load("operator/_discrete_operator.py", ["_n_conn_from_sections"], ns,
         class_name="DiscreteOperator")
    rng = np.random.default_rng(777)
    out = {}

    def flattened(packed, x_ids):
        sections = np.zeros(x_ids.shape[0], dtype=np.int64)
        xp, mels = ns["_get_conn_flattened_kernel"](
            x_ids, sections, packed["basis"], np.array(0.0), packed["diag_mels"],
            packed["n_conns"], packed["mels"], packed["x_prime"], packed["acting_on"],
            packed["acting_size"], packed["nonzero_diagonal"], False)
        return xp, sections

    def heis_terms(N, e, J):
        sz = np.array([[1.0, 0.0], [0.0, -1.0]])
        sx = np.array([[0.0, 1.0], [1.0, 0.0]])
        sy = np.array([[0.0, -1j], [1j, 0.0]])
        m = (np.kron(sz, sz) - np.kron(sx, sx) - np.real(np.kron(sy, sy))) * J
        return {tuple(sorted((int(i), int(j)))): m.real for i, j in e}

    cases = {
        "heis_chain10": (10, heis_terms(10, [(i, (i + 1) % 10) for i in range(10)], 1.0)),
        "ising_local_chain5": (5, None),
    }
    for name, (N, d) in cases.items():
        if d is None:
            e = edges["chain5"][:, :2]
            d = {(i,): -0.7 * oop.SIGMAX for i in range(5)}
            for i, j in e:
                d[(int(i), int(j))] = 1.3 * np.kron(oop.SIGMAZ, oop.SIGMAZ)
        packed = ns["pack_internals"](FakeHilbert(N), d, np.float64(0.0), np.float64, 1e-10)
        n = 64
        x_ids = rng.integers(0, 2, size=(n, N)).astype(np.int8)
        u = rng.random(n)
        vp, sections = flattened(packed, x_ids)
        prop = np.empty_like(x_ids)
        corr = np.zeros(n)
        ns["_choose"](vp, sections, u, prop, corr)
        _, sec2 = flattened(packed, prop)
        corr = corr - np.log(ns["_n_conn_from_sections"](sec2.copy()))
        out[name + "__x_ids"] = x_ids
        out[name + "__u"] = u
        out[name + "__proposed_ids"] = prop
        out[name + "__corr"] = corr
        out[name + "__aon"] = np.array([list(a) + [-1] * (2 - len(a)) for a in d])
        out[name + "__ops"] = np.array([np.pad(m, ((0, 4 - m.shape[0]), (0, 4 - m.shape[1])))
                                        for m in d.values()])
        out[name + "__sizes"] = np.array([len(a) for a in d])
        out[name + "__N"] = np.array(N)
    # IsingJax n_conn on +-1 states: h = 0.7, J = 1.3 and J = 0 (diagonal never counted)
    class StaticZero:
        pass
    ins = {"jnp": np, "jax": types.SimpleNamespace(jit=lambda f: f), "StaticZero": StaticZero}
    load("operator/_ising/jax.py", ["_ising_n_conn_jax"], ins)
    # open 7-site chain: 6 bonds, so J * sum(+-1) is zero for 3 domain walls
    e = np.array([(i, i + 1) for i in range(6)])
    x = rng.integers(0, 2, size=(200, 7)).astype(np.int8)
    out["ising_nconn__x_ids"] = x
    out["ising_nconn__edges"] = e
    out["ising_nconn__n"] = ins["_ising_n_conn_jax"](x, e, 0.7, 1.3)
    np.savez_compressed(os.path.join(HERE, "hamiltonian_rule.npz"), **out)


# ---------------------------------------------------------------- PauliStrings
class _DropKeyword(ast.NodeTransformer):
    """Remove a keyword argument numpy does not take (``promote_integers``)."""

    def __init__(self, name):
        self.name = name

    def visit_Call(self, node):
        self.generic_visit(node)
        node.keywords = [k for k in node.keywords if k.arg != self.name]
        return node


def gen_pauli_strings():
    """PauliStringsJax.get_conn_padded / n_conn (operator/_pauli_strings/jax.py:
    50-355) in its default "index" mode, on spin states."""
    import functools
    path = os.path.join(NK, "operator/_pauli_strings/jax.py")
    tree = ast.parse(open(path).read(), filename=path)
    names = ["_ising_conn_states_jax", "pack_internals", "sites_to_mask", "_check_mode",
             "pack_internals_jax", "_pauli_strings_mels_jax", "_pauli_strings_kernel_jax",
             "_pauli_strings_n_conn_jax"]
    nodes = [n for n in tree.body if isinstance(n, ast.FunctionDef) and n.name in names]
    assert {n.name for n in nodes} == set(names)
    for n in nodes:
        n.decorator_list = []
    mod = _DropKeyword("promote_integers").visit(ast.Module(body=nodes, type_ignores=[]))
    ast.fix_missing_locations(mod)
    jnp = types.SimpleNamespace(**{k: getattr(np, k) for k in dir(np) if not k.startswith("_")})
    jnp.bool_ = np.bool_
    jax = types.SimpleNamespace(lax=types.SimpleNamespace(select=np.where), jit=lambda f: f)
    ns = {"np": np, "jnp": jnp, "jax": jax, "partial": functools.partial,
          "_available_modes": ["index", "mask"]}
    exec(compile(mod, path, "exec"), ns)
    # the constructor's canonicalisation (canonicalize_input, _pauli_strings/base.py:
    # 61-137): duplicate strings summed (np.unique order), near-zero weights dropped
    load("operator/_pauli_strings/base.py", ["_reduce_pauli_string", "_remove_zero_weights"], ns)

    rng = np.random.default_rng(31)
    out = {}
    N = 10
    ring = [(i, (i + 1) % N) for i in range(N)]

    def pstr(ch):
        s = ["I"] * N
        for site, c in ch:
            s[site] = c
        return "".join(s)

    cases = {
        # TFIM written as strings: the ZZ strings share the empty flip set
        "tfim": ([pstr([(i, "X")]) for i in range(N)] +
                 [pstr([(i, "Z"), (j, "Z")]) for i, j in ring],
                 [-0.8] * N + [1.1] * N),
        # XX + YY + ZZ Heisenberg bonds: XX and YY share a flip set, so its
        # element is zero on aligned pairs (dropped by the cutoff)
        "heisenberg_xyz": ([pstr([(i, c), (j, c)]) for i, j in ring for c in "XYZ"],
                           [0.5, 0.5, 1.0] * N),
        # mixed strings: Y pairs, Z checks on flipped sites, long strings, a
        # repeated flip set with different weights, identity
        "mixed": (["XYIIIIIIYZ", "ZZZZZIIIII", "IIXXXXIIII", "YIYIIIIIIX", "XXXXXXXXXX",
                   "IIXXXXIIII", "IIIIIIIIII", "ZIIIIIIIIZ", "IXZYYZXIII", "YYYYIIIIII"],
                  [0.3, -1.25, 0.75, 0.5, -0.1, 0.25, 2.0, -0.6, 0.4, 1.5]),
    }
    cases["duplicates_and_zeros"] = (["ZZIIIIIIII", "XXIIIIIIII", "ZZIIIIIIII", "IYYIIIIIII",
                                      "XXIIIIIIII", "IIIIIIIIXX", "IIIIZIIIIZ"],
                                     [0.5, 1.0, 0.25, 2.0, -1.0, 1e-9, -0.75])
    for name, (ops, w) in cases.items():
        out[name + "__raw_ops"] = np.array(ops)
        out[name + "__raw_weights"] = np.array(w, dtype=np.float64)
        ops_a, w_a = ns["_reduce_pauli_string"](np.array(ops), np.array(w, dtype=np.float64))
        flips, z_data = ns["pack_internals_jax"](ops_a, w_a, weight_dtype=np.float64,
                                                 mode="index")
        x_ids = rng.integers(0, 2, size=(40, N)).astype(np.int8)
        xp_ids, mels, _ = ns["_pauli_strings_kernel_jax"](flips, z_data, x_ids, cutoff=1e-10)
        nconn = ns["_pauli_strings_n_conn_jax"](flips, z_data, x_ids, cutoff=1e-10)
        out[name + "__ops"] = ops_a
        out[name + "__weights"] = w_a
        out[name + "__x_ids"] = x_ids
        out[name + "__xp_ids"] = np.asarray(xp_ids, dtype=np.int8)
        out[name + "__mels"] = np.real(np.asarray(mels)).astype(np.float64)
        out[name + "__n_conn"] = np.asarray(nconn)
        out[name + "__flips"] = np.asarray(flips, dtype=np.int8)
    np.savez_compressed(os.path.join(HERE, "pauli_strings.npz"), **out)


def gen_hamiltonian_rule_pauli():
    """HamiltonianRuleJax.transition (sampler/rules/hamiltonian.py:166-213) over a
    PauliStringsJax operator, the operator's get_conn_padded / n_conn being the
    reference's own PauliStrings kernel functions; jax.random.randint is replaced
    by floor(u * maxval) for given uniforms u."""
    import functools
    path = os.path.join(NK, "operator/_pauli_strings/jax.py")
    tree = ast.parse(open(path).read(), filename=path)
    names = ["_ising_conn_states_jax", "pack_internals", "sites_to_mask", "_check_mode",
             "pack_internals_jax", "_pauli_strings_mels_jax", "_pauli_strings_kernel_jax",
             "_pauli_strings_n_conn_jax"]
    nodes = [n for n in tree.body if isinstance(n, ast.FunctionDef) and n.name in names]
    for n in nodes:
        n.decorator_list = []
    mod = _DropKeyword("promote_integers").visit(ast.Module(body=nodes, type_ignores=[]))
    ast.fix_missing_locations(mod)
    jnp = types.SimpleNamespace(**{k: getattr(np, k) for k in dir(np) if not k.startswith("_")})
    jnp.bool_ = np.bool_
    jax = types.SimpleNamespace(
        lax=types.SimpleNamespace(select=np.where), jit=lambda f: f,
        random=types.SimpleNamespace(
            randint=lambda key, shape, minval, maxval: np.floor(key * maxval).astype(np.int64)))
    ns = {"np": np, "jnp": jnp, "jax": jax, "partial": functools.partial,
          "_available_modes": ["index", "mask"]}
    exec(compile(mod, path, "exec"), ns)
    load("sampler/rules/hamiltonian.py", ["transition"], ns, class_name="HamiltonianRuleJax")

    N = 8
    ring = [(i, (i + 1) % N) for i in range(N)]

    def pstr(ch):
        s = ["I"] * N
        for site, c in ch:
            s[site] = c
        return "".join(s)

    ops = [pstr([(i, c), (j, c)]) for i, j in ring for c in "XYZ"] + [pstr([(0, "X")]),
                                                                      "XXXXIIII"]
    w = [0.5, 0.5, 1.0] * N + [-0.3, 0.4]
    flips, z_data = ns["pack_internals_jax"](np.array(ops), np.array(w), weight_dtype=np.float64,
                                             mode="index")

    class Op:
        def get_conn_padded(self, x):
            xp_ids, mels, _ = ns["_pauli_strings_kernel_jax"](flips, z_data, (1 - x) // 2,
                                                              cutoff=1e-10)
            return (1 - 2 * np.asarray(xp_ids)).astype(np.int8), np.real(mels)

        def n_conn(self, x):
            return ns["_pauli_strings_n_conn_jax"](flips, z_data, (1 - x) // 2, cutoff=1e-10)

    rule = types.SimpleNamespace(operator=Op())
    rng = np.random.default_rng(55)
    x = (1 - 2 * rng.integers(0, 2, size=(64, N))).astype(np.int8)
    u = rng.random(64)
    prop, corr = ns["transition"](rule, None, None, None, None, u, x)
    np.savez_compressed(os.path.join(HERE, "hamiltonian_rule_pauli.npz"), ops=np.array(ops),
                        weights=np.array(w), x=x, u=u, proposed=np.asarray(prop, dtype=np.int8),
                        corr=np.asarray(corr, dtype=np.float64))


# ---------------------------------------------------------------- log_cosh
def gen_logcosh():
    ns = {"jnp": np}
    load("nn/activation.py", ["log_cosh"], ns)
    x = np.concatenate([np.linspace(-30, 30, 601), np.array([0.0, -0.0, 1e-12, -1e-8, 50.0,
                                                               -700.0, 700.0])])
    rng = np.random.default_rng(7)
    x = np.concatenate([x, rng.normal(0, 2, 500)])
    np.savez_compressed(os.path.join(HERE, "logcosh.npz"), x=x, y=ns["log_cosh"](x))


# ---------------------------------------------------------------- stats
def gen_stats():
    jnp = types.SimpleNamespace(**{k: getattr(np, k) for k in dir(np) if not k.startswith("_")})
    jnp.clip = lambda a, lo=None, hi=None: np.clip(a, lo, hi)
    ns = {
        "np": np, "jnp": jnp, "jax": jax_stub,
        "nkjax": types.SimpleNamespace(dtype_real=lambda dt: np.float64),
        "config": types.SimpleNamespace(netket_use_plain_rhat=False),
        "Stats": lambda *a: np.array(a, dtype=np.float64),
    }
    load("stats/mc_stats_old.py", ["_get_blocks", "_block_variance", "_batch_variance",
                                   "_statistics"], ns)
    rng = np.random.default_rng(99)
    out = {}
    cases = {
        "c1": rng.normal(-20, 1.0, size=(16, 63)),
        "c2": rng.normal(-50, 3.0, size=(1024, 4)),
        "odd": rng.normal(0, 1, size=(40, 7)),
        "onechain": rng.normal(1, 1, size=(1, 100)),
        "wide": rng.normal(0, 1, size=(64, 64)),
    }
    # correlated chains (AR(1)) so that tau > 0 and the block path is exercised
    ar = np.zeros((8, 1024))
    for t in range(1, 1024):
        ar[:, t] = 0.95 * ar[:, t - 1] + rng.normal(size=8)
    cases["ar1_blocks"] = ar
    cases["ar1_slow"] = np.cumsum(rng.normal(size=(40, 64)), axis=1)
    for k, v in cases.items():
        out[k + "__data"] = v
        out[k + "__stats"] = ns["_statistics"](v, 32)
    np.savez_compressed(os.path.join(HERE, "stats.npz"), **out)


# ---------------------------------------------------------------- NGD
def _ngd_namespace():
    """The reference's NGD update functions and solvers on numpy stand-ins."""
    jnp = types.SimpleNamespace(**{k: getattr(np, k) for k in dir(np) if not k.startswith("_")})
    # XLA's factorisations return NaN instead of raising; mirror that
    def cho_factor(A, lower=False):
        try:
            return scipy.linalg.cho_factor(A, lower=lower, check_finite=False)
        except np.linalg.LinAlgError:
            return np.full_like(A, np.nan), lower

    def cho_solve(cl, b):
        return scipy.linalg.cho_solve(cl, b, check_finite=False)

    def eigh(A):
        if not np.all(np.isfinite(A)):
            return np.full(A.shape[0], np.nan), np.full_like(A, np.nan)
        return np.linalg.eigh(A)

    jnp.linalg = types.SimpleNamespace(eigh=eigh)
    jsp = types.SimpleNamespace(linalg=types.SimpleNamespace(cho_factor=cho_factor,
                                                             cho_solve=cho_solve))
    ns = {"np": np, "jnp": jnp, "jax": jax_stub, "jsp": jsp,
          "ravel_pytree": ravel_identity,
          "config": types.SimpleNamespace(netket_sharding=False),
          "nkjax": types.SimpleNamespace(tree_leaf_iscomplex=lambda s: False),
          "ensure_accepts_kwargs": lambda f, *names: (lambda A, b, **kw: f(A, b)),
          "warn_deprecation": lambda *a, **k: None,
          "Union": object}
    load("_src/ngd/sr_srt_common.py", ["_prepare_input"], ns)
    load("_src/ngd/srt.py", ["_compute_srt_update"], ns)
    load("_src/ngd/sr.py", ["_compute_sr_update"], ns)
    load("optimizer/solver/solvers.py", ["cholesky", "pinv_smooth", "cholesky_with_fallback"], ns)
    load("_src/solvers/nan_fallback.py", ["_nan_fallback_solver"], ns)
    # cholesky_with_fallback builds pinv_smooth(rtol=..) through partial_from_kwargs;
    # restore that behaviour for keyword-only calls
    pinv = ns["pinv_smooth"]

    def pinv_kw(A=None, b=None, **kw):
        if A is None:
            return lambda A_, b_, x0=None: pinv(A_, b_, **kw)
        return pinv(A, b, **kw)
    ns["pinv_smooth"] = pinv_kw
    return ns


def gen_ngd():
    ns = _ngd_namespace()
    rng = np.random.default_rng(2024)
    out = {}
    for name, n, P, shift in [("minsr", 48, 120, 1e-4), ("sr", 96, 40, 1e-2),
                              ("minsr_big_shift", 32, 64, 0.1)]:
        O = rng.normal(size=(n, P))
        O = O - O.mean(axis=0)
        e = rng.normal(-3, 1, size=n)
        O_L, dv = ns["_prepare_input"](O, e, mode="real", scaling_factor=1.0 / n)
        solver = ns["cholesky_with_fallback"]
        if name.startswith("minsr"):
            upd, _, info = ns["_compute_srt_update"](O_L, dv, diag_shift=shift,
                                                     solver_fn=solver, mode="real",
                                                     params_structure=None)
        else:
            upd, _, info = ns["_compute_sr_update"](O_L, dv, diag_shift=shift,
                                                    solver_fn=solver, mode="real",
                                                    params_structure=None)
        out[name + "__O"] = O
        out[name + "__e"] = e
        out[name + "__shift"] = np.array(shift)
        out[name + "__update"] = np.asarray(upd)
        out[name + "__fallback"] = np.array(bool(info["solver_fallback"]))
    # fallback: NaN in the matrix routes to pinv_smooth
    A = rng.normal(size=(12, 12))
    A = A @ A.T + 1e-3 * np.eye(12)
    b = rng.normal(size=12)
    x, info = ns["cholesky_with_fallback"](A, b)
    out["solve_spd__A"], out["solve_spd__b"], out["solve_spd__x"] = A, b, np.asarray(x)
    Ab = A.copy()
    Ab[0, 0] = np.nan
    xb, infob = ns["cholesky_with_fallback"](Ab, b)
    out["solve_nan__x"] = np.asarray(xb)
    out["solve_nan__fallback"] = np.array(bool(infob["solver_fallback"]))
    # singular matrix: pinv_smooth directly
    U = rng.normal(size=(10, 4))
    S = U @ U.T
    xs, _ = ns["pinv_smooth"](S, b[:10])
    out["pinv_singular__A"], out["pinv_singular__b"], out["pinv_singular__x"] = S, b[:10], xs
    np.savez_compressed(os.path.join(HERE, "ngd.npz"), **out)


# ---------------------------------------------------------------- SPRING
def gen_spring():
    """_compute_srt_update / _compute_sr_update with momentum, old_updates and
    proj_reg (_src/ngd/srt.py:22-96, _src/ngd/sr.py:23-80): SPRING."""
    ns = _ngd_namespace()
    rng = np.random.default_rng(77)
    out = {}
    cases = [("srt_momentum", "srt", 48, 120, 1e-4, None, 0.8),
             ("srt_proj", "srt", 48, 120, 1e-4, 0.5, None),
             ("srt_both", "srt", 40, 96, 1e-3, 1.0, 0.9),
             ("sr_momentum", "sr", 96, 40, 1e-2, None, 0.8)]
    for name, kind, n, P, shift, proj, mom in cases:
        O = rng.normal(size=(n, P))
        O = O - O.mean(axis=0)
        e = rng.normal(-3, 1, size=n)
        old = rng.normal(scale=0.1, size=P)
        O_L, dv = ns["_prepare_input"](O, e, mode="real", scaling_factor=1.0 / n)
        f = ns["_compute_srt_update"] if kind == "srt" else ns["_compute_sr_update"]
        upd, new_old, info = f(O_L, np.array(dv), diag_shift=shift,
                               solver_fn=ns["cholesky_with_fallback"], mode="real",
                               proj_reg=proj, momentum=mom,
                               old_updates=None if mom is None else old,
                               params_structure=None)
        out[name + "__O"], out[name + "__e"], out[name + "__old"] = O, e, old
        out[name + "__cfg"] = np.array([shift, -1.0 if proj is None else proj,
                                        -1.0 if mom is None else mom])
        out[name + "__update"] = np.asarray(upd)
        out[name + "__new_old"] = (np.zeros(0) if new_old is None else np.asarray(new_old))
    np.savez_compressed(os.path.join(HERE, "spring.npz"), **out)


# ---------------------------------------------------------------- online stats
class AtArray(np.ndarray):
    """ndarray with jax's functional ``x.at[idx].add(v)``."""

    @property
    def at(self):
        arr = self

        class _Idx:
            def __getitem__(self, idx):
                class _Op:
                    def add(self, v):
                        out = np.array(arr, copy=True).view(AtArray)
                        out[idx] += v
                        return out
                return _Op()
        return _Idx()


def lax_scan(f, init, xs):
    carry = init
    for x in xs:
        carry, _ = f(carry, x)
    return carry, None


def lax_dynamic_slice_in_dim(a, start, size, axis=0):
    # XLA clamps the start index so that the slice stays in bounds
    start = int(min(max(int(start), 0), a.shape[axis] - size))
    idx = [slice(None)] * a.ndim
    idx[axis] = slice(start, start + size)
    return a[tuple(idx)]


def gen_online_stats():
    jnp = types.SimpleNamespace(**{k: getattr(np, k) for k in dir(np) if not k.startswith("_")})
    jax = types.SimpleNamespace(
        jit=lambda *a, **k: (lambda f: f),
        lax=types.SimpleNamespace(scan=lax_scan, dynamic_slice_in_dim=lax_dynamic_slice_in_dim))
    ns = {"np": np, "jnp": jnp, "jax": jax, "lax": jax.lax,
          "partial": lambda *a, **k: (lambda f: f)}
    load("_src/stats/online_stats/kernels.py", ["_acf_core", "_update_arrays"], ns)
    import math
    gns = {"np": np, "jnp": jnp, "jax": jax, "isnan": math.isnan, "sqrt": math.sqrt,
           "_NaN": np.nan,
           "Stats": lambda **kw: np.array([kw["mean"], kw["error_of_mean"], kw["variance"],
                                           kw["tau_corr"], kw["R_hat"]], dtype=np.float64)}
    getters = ["mean", "variance", "tau_corr", "tau_corr_batch", "tau_corr_acf", "acf",
               "R_hat", "n_chains", "get_stats", "_compute_error_of_mean"]
    load("_src/stats/online_stats/accumulator.py", getters, gns, class_name="OnlineStats")
    props = {g: property(gns[g]) for g in getters if g not in ("get_stats",
                                                               "_compute_error_of_mean")}
    props["get_stats"] = gns["get_stats"]
    props["_compute_error_of_mean"] = gns["_compute_error_of_mean"]
    FakeOS = type("FakeOS", (), props)

    def run(chunks, max_lag, decay):
        C = chunks[0].shape[0]
        acf_len = max_lag + 1 if max_lag > 0 else 0
        z = lambda *s: np.zeros(s).view(AtArray)
        st = [z(C), np.zeros(C), z(C), z(C, acf_len), z(C, acf_len), z(C, acf_len),
              z(C, acf_len), z(C, max_lag)]
        buf_len, n_total = 0, 0
        for d in chunks:
            st = list(ns["_update_arrays"](*st, decay, max_lag, buf_len, d))
            st = [np.asarray(a).view(AtArray) for a in st]
            buf_len = min(buf_len + d.shape[1], max_lag)
            n_total += d.size
        o = FakeOS()
        (o._chain_count, o._chain_mean, o._chain_M2, o._cross_sum, o._m1_sum, o._m2_sum,
         o._pair_count, o._chain_buf) = [np.asarray(a) for a in st]
        o.max_lag, o._n_samples_total, o._buf_len = max_lag, n_total, buf_len
        derived = np.array([o.mean, o.variance, o.tau_corr, o.tau_corr_batch,
                            o.tau_corr_acf, o.R_hat, float(np.real(o.get_stats()[1]))],
                           dtype=np.float64)
        acf = o.acf
        return [np.asarray(a) for a in st], buf_len, derived, (
            np.zeros(0) if acf is None else np.asarray(acf))

    rng = np.random.default_rng(2024)

    def ar1(C, T, phi):
        x = np.zeros((C, T))
        x[:, 0] = rng.standard_normal(C)
        for t in range(1, T):
            x[:, t] = phi * x[:, t - 1] + math.sqrt(1 - phi ** 2) * rng.standard_normal(C)
        return x

    cases = {
        # (chunk lengths along the chain axis, n_chains, max_lag, decay, generator)
        "iid_oneshot": ([300], 8, 64, None, "iid"),
        "iid_chunks": ([30] * 10, 8, 32, None, "iid"),
        "ar1_small_batches": ([4] * 40, 16, 64, None, "ar1"),
        "ar1_ragged": ([1, 7, 3, 64, 2, 100, 5], 6, 16, None, "ar1"),
        "big_then_small": ([12, 6, 6, 6, 6, 6], 4, 8, None, "iid"),
        "decay": ([50] * 6, 4, 16, 0.9, "ar1"),
        "no_acf": ([40] * 5, 6, 0, None, "iid"),
        "one_chain": ([200, 56], 1, 64, None, "ar1"),
        "shifted_mean": ([5] * 20, 64, 64, None, "shift"),
    }
    out = {}
    for name, (lens, C, max_lag, decay, gen) in cases.items():
        T = sum(lens)
        if gen == "iid":
            data = rng.standard_normal((C, T))
        elif gen == "ar1":
            data = ar1(C, T, 0.8)
        else:
            data = -37.5 + 0.25 * rng.standard_normal((C, T))
        chunks = np.split(data, np.cumsum(lens)[:-1], axis=1)
        st, buf_len, derived, acf = run(chunks, max_lag, decay)
        out[name + "__data"] = data
        out[name + "__lens"] = np.array(lens)
        out[name + "__cfg"] = np.array([max_lag, -1.0 if decay is None else decay])
        for key, a in zip(["count", "mean", "M2", "cross", "m1", "m2", "pair", "buf"], st):
            out[f"{name}__{key}"] = a
        out[name + "__buf_len"] = np.array(buf_len)
        out[name + "__derived"] = derived
        out[name + "__acf"] = acf
    np.savez_compressed(os.path.join(HERE, "online_stats.npz"), **out)


def gen_pauli_products():
    """PauliStrings @ PauliStrings for real weights (operator/_pauli_strings/
    base.py:330-371, 501-660): the product string and phase per pair of strings,
    op1-major pair order, then the duplicate reduction; and the predicate that
    makes the reference switch to complex weights (an odd number of Y in some
    product string)."""
    import itertools
    ns = {"np": np, "product": itertools.product,
          "nkjax": types.SimpleNamespace(
              is_complex_dtype=lambda d: np.issubdtype(np.dtype(d), np.complexfloating))}
    load("operator/_pauli_strings/base.py",
         ["_pauli_to_num", "_num_to_pauli", "_levi_term", "_apply_pauli_op_reduction",
          "_split_string", "_make_new_pauli_string", "_remove_zero_weights",
          "_reduce_pauli_string", "_will_matmul_produce_complex_coefficients", "_matmul"], ns)
    rng = np.random.default_rng(47)
    N = 6

    def real_strings(k):
        out = []
        while len(out) < k:
            s = "".join(rng.choice(list("IXYZ"), size=N))
            if s.count("Y") % 2 == 0:
                out.append(s)
        return out

    cases = {
        "xx_yy": (["XXIIII", "YYIIII"], [1.0, 1.0], ["XXIIII", "YYIIII"], [1.0, -1.0]),
        "square": (["ZZIIII", "XIIIII", "IXIIII"], [0.5, -1.0, 0.25],
                   ["ZZIIII", "XIIIII", "IXIIII"], [0.5, -1.0, 0.25]),
        "heis_bonds": (["XXIIII", "YYIIII", "ZZIIII"], [1.0, 1.0, 1.0],
                       ["IXXIII", "IYYIII", "IZZIII"], [1.0, 1.0, 1.0]),
        "complex_xz": (["XIIIII"], [1.0], ["ZIIIII"], [1.0]),
    }
    for k in range(6):
        na, nb = int(rng.integers(1, 6)), int(rng.integers(1, 6))
        cases[f"random{k}"] = (real_strings(na), list(rng.normal(size=na)),
                               real_strings(nb), list(rng.normal(size=nb)))

    def strings_from(alphabet, k):
        return ["".join(rng.choice(list(alphabet), size=N)) for _ in range(k)]

    # products that stay real: X/I strings, Z/I strings, YY pairs with X/I
    # elsewhere, and a symmetric square whose imaginary cross terms cancel
    for k in range(3):
        na, nb = int(rng.integers(2, 6)), int(rng.integers(2, 6))
        cases[f"x_only{k}"] = (strings_from("IX", na), list(rng.normal(size=na)),
                               strings_from("IX", nb), list(rng.normal(size=nb)))
        cases[f"z_only{k}"] = (strings_from("IZ", na), list(rng.normal(size=na)),
                               strings_from("IZ", nb), list(rng.normal(size=nb)))
        ya = ["YY" + s[2:] for s in strings_from("IX", na)]
        yb = ["YY" + s[2:] for s in strings_from("IX", nb)]
        cases[f"yy_pairs{k}"] = (ya, list(rng.normal(size=na)), yb, list(rng.normal(size=nb)))
        sq = strings_from("IXZ", na)
        wq = list(rng.normal(size=na))
        cases[f"square{k}"] = (sq, wq, sq, wq)
    out = {}
    for name, (a_ops, a_w, b_ops, b_w) in cases.items():
        ao, aw = ns["_reduce_pauli_string"](np.array(a_ops), np.array(a_w, dtype=np.float64))
        bo, bw = ns["_reduce_pauli_string"](np.array(b_ops), np.array(b_w, dtype=np.float64))
        cplx = bool(ns["_will_matmul_produce_complex_coefficients"](ao, bo))
        out[name + "__a_ops"], out[name + "__a_w"] = np.array(a_ops), np.array(a_w, np.float64)
        out[name + "__b_ops"], out[name + "__b_w"] = np.array(b_ops), np.array(b_w, np.float64)
        out[name + "__complex"] = np.array(cplx)
        dtype = np.complex128 if cplx else np.float64
        ops, w = ns["_matmul"](ao, aw.astype(dtype), bo, bw.astype(dtype), dtype=dtype)
        out[name + "__ops"] = np.asarray(ops)
        out[name + "__weights"] = np.asarray(w)
    np.savez_compressed(os.path.join(HERE, "pauli_products.npz"), **out)


def gen_stats_format():
    """Stats printing: _format_main_string / _format_scientific_notation
    (stats/mc_stats.py:26-74) on means and errors spanning the branches (large
    and small values, tiny errors, zero error, non-finite)."""
    import math
    ns = {"np": np, "math": math}
    load("stats/mc_stats.py", ["_format_main_string", "_format_scientific_notation"], ns)
    rng = np.random.default_rng(5)
    rows = [(-10.2516, 0.0123, 0.5), (1e-4, 2.3e-6, 1e-9), (3.0, 0.0, 0.0),
            (float("nan"), float("nan"), float("nan")), (-43.88123, 0.00071, 1.7),
            (0.5, 1e-8, 1e-12), (123456.7, 89.1, 3e4), (-2e-3, 4e-3, 1e-5), (1.0, 1e-16, 0.0),
            (float("inf"), 0.1, 1.0), (-7.25, 2.5, 6.0)]
    for _ in range(20):
        rows.append((float(rng.normal() * 10.0 ** rng.integers(-5, 5)),
                     float(abs(rng.normal()) * 10.0 ** rng.integers(-9, 2)),
                     float(abs(rng.normal()))))
    vals = np.array(rows, dtype=np.float64)
    strs = np.array([ns["_format_main_string"](*r) for r in rows])
    np.savez_compressed(os.path.join(HERE, "stats_format.npz"), values=vals, strings=strs)


if __name__ == "__main__":
    edges = gen_edges()
    gen_ising(edges)
    gen_localop(edges)
    gen_logcosh()
    gen_stats()
    gen_online_stats()
    gen_hamiltonian_rule(edges)
    gen_hamiltonian_rule_pauli()
    gen_ngd()
    gen_spring()
    gen_pauli_products()
    gen_lattice_edges()
    gen_stats_format()
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)), "bytes")
