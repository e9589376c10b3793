"""Pin the CPU oracle against golden vectors produced by NetKet's own source
(tests/golden/make_golden.py)."""
import numpy as np
import pytest

from oracle import graph as og
from oracle import hilbert as oh
from oracle import operator as oop
from oracle import rbm as orbm
from oracle import stats as ost
from oracle import ngd as ongd

EDGE_CASES = ["chain16", "chain5", "chain8_obc", "chain14_nnn", "square4", "square6_nnn",
              "square10_nnn", "square16", "cube3"]


@pytest.mark.parametrize("name", EDGE_CASES)
def test_edges_match_reference_order(golden, name):
    g = golden("edges")
    meta = g[name + "__meta"]
    extent, pbc, order = list(meta[:-2]), bool(meta[-2]), int(meta[-1])
    mine = np.array(og.lattice_edges(extent, pbc, order), dtype=np.int64).reshape(-1, 3)
    np.testing.assert_array_equal(mine, g[name])


@pytest.mark.parametrize("name", ["chain16", "chain5", "square4"])
def test_ising_conn_matches_numba_kernel(golden, name):
    gi = golden("ising")
    edges = golden("edges")[name][:, :2]
    h, J = gi[name + "__hJ"]
    x = oh.local_indices_to_states(gi[name + "__x_ids"])
    xp, mels = oop.ising_get_conn_padded(x, edges, h, J)
    n, K, N = xp.shape
    ref_xp = oh.local_indices_to_states(gi[name + "__xp_ids"]).reshape(n, K, N)
    np.testing.assert_array_equal(xp, ref_xp)
    np.testing.assert_array_equal(mels, gi[name + "__mels"].reshape(n, K))


LOCALOP_CASES = ["heis_chain16", "heis_square4", "heis_square4_nosign", "j1j2_square6",
                 "j1j2_chain14", "j1j2_square10", "ising_local_chain5"]


def _build_local(gl, name, golden):
    N = int(gl[name + "__N"])
    ops, aon = [], []
    for a, m, s in zip(gl[name + "__aon"], gl[name + "__ops"], gl[name + "__sizes"]):
        d = 2**int(s)
        ops.append(m[:d, :d])
        aon.append([int(v) for v in a[:s]])
    return N, oop.LocalOperator(N, ops, aon)


def _heis_from_graph(golden, name):
    table = {"heis_chain16": ("chain16", 1.0, None), "heis_square4": ("square4", 1.0, None),
             "heis_square4_nosign": ("square4", 1.0, False),
             "j1j2_square6": ("square6_nnn", [1.0, 0.5], None),
             "j1j2_chain14": ("chain14_nnn", [1.0, 0.2], None),
             "j1j2_square10": ("square10_nnn", [1.0, 0.5], None)}
    gname, J, sr = table[name]
    ge = golden("edges")
    meta = ge[gname + "__meta"]
    N = int(np.prod(meta[:-2]))
    g = og.Graph([tuple(r) for r in ge[gname]], N)
    return oop.heisenberg(N, g, J, sign_rule=sr)


@pytest.mark.parametrize("name", LOCALOP_CASES)
def test_localop_terms_match_reference_construction(golden, name):
    """Heisenberg/GraphOperator term order and matrices equal NetKet's."""
    if name == "ising_local_chain5":
        pytest.skip("built directly from terms")
    gl = golden("localop")
    op = _heis_from_graph(golden, name)
    assert [list(a) for a in op.acting_on] == [list(a[:s]) for a, s in
                                               zip(gl[name + "__aon"], gl[name + "__sizes"])]
    for m, ref in zip(op.operators, gl[name + "__ops"]):
        np.testing.assert_array_equal(m, ref[:m.shape[0], :m.shape[1]])


@pytest.mark.parametrize("name", LOCALOP_CASES)
def test_localop_conn_matches_numba_kernel(golden, name):
    gl = golden("localop")
    N, op = _build_local(gl, name, golden)
    assert op.max_conn_size == int(gl[name + "__max_conn_jax"])
    x = oh.local_indices_to_states(gl[name + "__x_ids"])
    sections = gl[name + "__sections"]
    ref_xp = oh.local_indices_to_states(gl[name + "__xp_ids"])
    ref_m = gl[name + "__mels"]
    # numba order, unfiltered, per sample
    flat = op.get_conn_flattened_numba_order(x)
    start = 0
    for b, (xs, ms) in enumerate(flat):
        stop = sections[b]
        np.testing.assert_array_equal(xs, ref_xp[start:stop])
        np.testing.assert_array_equal(ms, ref_m[start:stop])
        start = stop
    # padded JAX order == numba order with |mel| <= cutoff dropped, when all
    # terms act on the same number of sites (one group)
    xp, mels = op.get_conn_padded(x)
    single_group = len(set(gl[name + "__sizes"].tolist())) == 1
    start = 0
    for b in range(x.shape[0]):
        stop = sections[b]
        keep = np.abs(ref_m[start:stop]) > 1e-10
        rx, rm = ref_xp[start:stop][keep], ref_m[start:stop][keep]
        k = len(rm)
        if single_group:
            np.testing.assert_array_equal(xp[b, :k], rx)
            np.testing.assert_array_equal(mels[b, :k], rm)
        else:  # canonicalised comparison (test/operator/test_hamiltonian.py:160-218)
            o1 = np.lexsort(xp[b, :k].T)
            o2 = np.lexsort(rx.T)
            np.testing.assert_array_equal(xp[b, :k][o1], rx[o2])
            np.testing.assert_array_equal(mels[b, :k][o1], rm[o2])
        assert np.all(mels[b, k:] == 0)
        assert np.all(xp[b, k:] == x[b])
        start = stop


def test_log_cosh(golden):
    g = golden("logcosh")
    np.testing.assert_array_equal(orbm.log_cosh(g["x"]), g["y"])


@pytest.mark.parametrize("name", ["c1", "c2", "odd", "onechain", "wide", "ar1_blocks",
                                  "ar1_slow"])
def test_stats(golden, name):
    g = golden("stats")
    s = ost.statistics(g[name + "__data"]).as_array()
    np.testing.assert_allclose(s, g[name + "__stats"], rtol=1e-12, atol=1e-14,
                               equal_nan=True)


@pytest.mark.parametrize("name", ["minsr", "sr", "minsr_big_shift"])
def test_ngd_updates(golden, name):
    g = golden("ngd")
    O, e, shift = g[name + "__O"], g[name + "__e"], float(g[name + "__shift"])
    if name.startswith("minsr"):
        upd, info = ongd.srt_update(O, e, shift)
    else:
        upd, info = ongd.sr_update(O, e, shift)
    np.testing.assert_allclose(upd, g[name + "__update"], rtol=1e-10, atol=1e-12)
    assert info["solver_fallback"] == bool(g[name + "__fallback"])


def test_solvers(golden):
    g = golden("ngd")
    x, info = ongd.cholesky_with_fallback(g["solve_spd__A"], g["solve_spd__b"])
    np.testing.assert_allclose(x, g["solve_spd__x"], rtol=1e-12)
    assert not info["solver_fallback"]
    A = g["solve_spd__A"].copy()
    A[0, 0] = np.nan
    _, info = ongd.cholesky_with_fallback(A, g["solve_spd__b"])
    assert info["solver_fallback"] and bool(g["solve_nan__fallback"])
    xs, _ = ongd.pinv_smooth(g["pinv_singular__A"], g["pinv_singular__b"])
    np.testing.assert_allclose(xs, g["pinv_singular__x"], rtol=1e-8, atol=1e-10)


def test_minsr_equals_sr():
    """Woodbury identity, as NetKet's test/driver/test_srt.py:98-175 (atol 1e-10)."""
    rng = np.random.default_rng(0)
    O = rng.normal(size=(40, 25))
    O -= O.mean(0)
    e = rng.normal(size=40)
    a, _ = ongd.srt_update(O, e, 1e-3)
    b, _ = ongd.sr_update(O, e, 1e-3)
    np.testing.assert_allclose(a, b, atol=1e-10)


@pytest.mark.parametrize("name", ["heis_square4", "j1j2_square6", "j1j2_square10"])
def test_vectorised_conn_equals_loop_oracle(golden, name):
    from oracle import vmc_step
    gl = golden("localop")
    N, op = _build_local(gl, name, golden)
    rng = np.random.default_rng(5)
    x = oh.local_indices_to_states(rng.integers(0, 2, size=(40, N)))
    xp, m = vmc_step.conn_two_site(x, vmc_step.two_site_tables(op))
    rxp, rm = op.get_conn_padded(x)
    np.testing.assert_array_equal(xp, rxp)
    np.testing.assert_array_equal(m, rm)


ONLINE_CASES = ["iid_oneshot", "iid_chunks", "ar1_small_batches", "ar1_ragged",
                "big_then_small", "decay", "no_acf", "one_chain", "shifted_mean"]


def online_oracle_run(g, name):
    from oracle import online_stats as oos
    data, lens, cfg = g[name + "__data"], g[name + "__lens"], g[name + "__cfg"]
    decay = None if cfg[1] < 0 else float(cfg[1])
    s = oos.new_state(data.shape[0], int(cfg[0]))
    for ch in np.split(data, np.cumsum(lens)[:-1], axis=1):
        s = oos.update(s, ch, decay)
    return s


def acf_tolerance(g, name):
    """The ACF is formed from raw moment sums (sum x_t x_{t-k} - sum x_{t-k} sum
    x_t / n), so rounding in the sums is amplified by mean^2 / variance."""
    d = g[name + "__data"]
    return 1e-13 * max(1.0, float(np.mean(d)) ** 2 / float(np.var(d)))


@pytest.mark.parametrize("name", ONLINE_CASES)
def test_online_stats_oracle(golden, name):
    """Oracle restatement of OnlineStats vs the reference's own _update_arrays /
    _acf_core and read-outs, executed on the same chunks."""
    from oracle import online_stats as oos
    g = golden("online_stats")
    s = online_oracle_run(g, name)
    for k in ("count", "mean", "M2", "cross", "m1", "m2", "pair", "buf"):
        ref = g[f"{name}__{k}"]
        scale = max(1.0, float(np.abs(ref).max())) if ref.size else 1.0
        np.testing.assert_allclose(s[k], ref, rtol=0, atol=1e-14 * scale, err_msg=k)
    assert s["buf_len"] == int(g[name + "__buf_len"])
    np.testing.assert_allclose(oos.derived(s), g[name + "__derived"], rtol=1e-11,
                               atol=1e-13, equal_nan=True)
    a, ga = oos.acf(s), g[name + "__acf"]
    if ga.size == 0:
        assert a is None
    else:
        np.testing.assert_allclose(a, ga, rtol=0, atol=acf_tolerance(g, name))


@pytest.mark.parametrize("name", ["heis_chain10", "ising_local_chain5"])
def test_hamiltonian_rule_proposal(golden, name):
    """Oracle Hamiltonian-rule proposal vs the reference's numba transition
    (get_conn_flattened, _choose, n_conn) on the same states and uniforms."""
    from oracle import hilbert as oh_
    from oracle import sampler as osamp
    g = golden("hamiltonian_rule")
    N = int(g[name + "__N"])
    ops = [m[:2 ** s, :2 ** s] for m, s in zip(g[name + "__ops"], g[name + "__sizes"])]
    aon = [list(a[:s]) for a, s in zip(g[name + "__aon"], g[name + "__sizes"])]
    op = oop.LocalOperator(N, ops, aon)
    x = oh_.local_indices_to_states(g[name + "__x_ids"])
    prop, corr = osamp.hamiltonian_propose(op, x, g[name + "__u"], diag_rule=1)
    np.testing.assert_array_equal(prop, oh_.local_indices_to_states(g[name + "__proposed_ids"]))
    np.testing.assert_allclose(corr, g[name + "__corr"], rtol=0, atol=1e-15)


def test_hamiltonian_rule_ising_count(golden):
    """diag_rule 2 on Ising's LocalOperator tables counts IsingJax's n_conn:
    N flips plus the diagonal only where J * sum(+-1) != 0."""
    from oracle import hilbert as oh_
    from oracle import sampler as osamp
    g = golden("hamiltonian_rule")
    x = oh_.local_indices_to_states(g["ising_nconn__x_ids"])
    op = oop.ising_as_local_operator(7, g["ising_nconn__edges"], 0.7, 1.3)
    n = [len(r) for r in osamp.hamiltonian_row(op, x, diag_rule=2)]
    np.testing.assert_array_equal(n, g["ising_nconn__n"])
    assert set(g["ising_nconn__n"]) == {7, 8}


@pytest.mark.parametrize("name", ["tfim", "heisenberg_xyz", "mixed", "duplicates_and_zeros"])
def test_pauli_strings_canonicalize(golden, name):
    """The constructor's reduction of the raw strings equals the reference's
    _reduce_pauli_string (duplicates summed, sorted, near-zero weights dropped)."""
    g = golden("pauli_strings")
    ops, w = oop.pauli_canonicalize(list(g[name + "__raw_ops"]), g[name + "__raw_weights"])
    assert list(ops) == list(g[name + "__ops"])
    np.testing.assert_array_equal(w, g[name + "__weights"])


@pytest.mark.parametrize("name", ["tfim", "heisenberg_xyz", "mixed", "duplicates_and_zeros"])
def test_pauli_strings_conn(golden, name):
    """Oracle PauliStrings get_conn_padded / n_conn vs the reference's own
    pack_internals_jax + _pauli_strings_kernel_jax (index mode)."""
    from oracle import hilbert as oh_
    g = golden("pauli_strings")
    x = oh_.local_indices_to_states(g[name + "__x_ids"])
    xp, mels, nc = oop.pauli_get_conn_padded(x, list(g[name + "__raw_ops"]),
                                             g[name + "__raw_weights"])
    np.testing.assert_array_equal(xp, oh_.local_indices_to_states(g[name + "__xp_ids"]))
    np.testing.assert_array_equal(mels, g[name + "__mels"])
    np.testing.assert_array_equal(nc, g[name + "__n_conn"])


@pytest.mark.parametrize("name", ["srt_momentum", "srt_proj", "srt_both", "sr_momentum"])
def test_spring_updates(golden, name):
    """Oracle SR / minSR with SPRING momentum and proj_reg vs the reference's own
    _compute_srt_update / _compute_sr_update."""
    g = golden("spring")
    shift, proj, mom = g[name + "__cfg"]
    proj = None if proj < 0 else float(proj)
    mom = None if mom < 0 else float(mom)
    f = ongd.srt_update if name.startswith("srt") else ongd.sr_update
    kw = {"proj_reg": proj} if name.startswith("srt") else {}
    if mom is not None:
        kw.update(momentum=mom, old_updates=g[name + "__old"])
    res = f(g[name + "__O"], g[name + "__e"], float(shift), **kw)
    np.testing.assert_allclose(res[0], g[name + "__update"], rtol=1e-10, atol=1e-12)
    if mom is not None:
        np.testing.assert_allclose(res[2], g[name + "__new_old"], rtol=1e-10, atol=1e-12)


@pytest.mark.parametrize("ham", ["ising", "heisenberg"])
def test_full_sum_gradient_equals_finite_differences(ham):
    """The gradient formula 2 Re<(O - <O>) (E_loc - E)> (netket/vqs/mc/common.py:
    103-118) equals central finite differences of the exact energy <psi|H|psi>/
    <psi|psi> (the reference's own check, test/variational/test_variational.py:
    362-414), here on the oracle for a 6-site RBM."""
    from oracle import exact as oex
    N = 6
    rng = np.random.default_rng(17)
    p = orbm.init_params(rng, N, alpha=2, std=0.3)
    flat0 = orbm.ravel(p)
    M = len(p["bias"])
    edges = np.array([(i, (i + 1) % N) for i in range(N)])
    if ham == "ising":
        conn = lambda s: oop.ising_get_conn_padded(s, edges, 0.8, 1.1)
        tsz = None
    else:
        op = oop.heisenberg(N, og.Graph([(int(i), int(j), 0) for i, j in edges], N), 1.0, None)
        conn = op.get_conn_padded
        tsz = 0
    E, G = oex.full_sum_energy_and_grad(p, conn, N, tsz)
    h = 1e-5
    fd = np.empty_like(flat0)
    for k in range(flat0.size):
        f = flat0.copy()
        f[k] += h
        Ep, _ = oex.full_sum_energy_and_grad(orbm.unravel(f, N, M), conn, N, tsz)
        f[k] -= 2 * h
        Em, _ = oex.full_sum_energy_and_grad(orbm.unravel(f, N, M), conn, N, tsz)
        fd[k] = (Ep - Em) / (2 * h)
    np.testing.assert_allclose(G, fd, rtol=1e-6, atol=1e-8)


@pytest.mark.parametrize("N,h,J", [(8, 1.0, 1.0), (10, 0.5, 1.0), (12, 1.7, -0.8)])
def test_ed_matches_free_fermion_tfim(N, h, J):
    """Lanczos ground energy of the oracle's sparse TFIM (get_conn -> sparse H)
    equals the Jordan-Wigner closed form on the ring (even parity sector, even N)."""
    from oracle import exact as oex
    edges = np.array([(i, (i + 1) % N) for i in range(N)])
    E0 = oex.lanczos_ed(lambda s: oop.ising_get_conn_padded(s, edges, h, J), N)[0]
    np.testing.assert_allclose(E0, oex.tfim_ground_energy(N, J, h), rtol=1e-10)


def test_hamiltonian_rule_pauli_proposal(golden):
    """Oracle PauliStrings Hamiltonian-rule proposal vs the reference's own
    HamiltonianRuleJax.transition over its PauliStrings kernel, with the same
    uniforms (rand_i = floor(u n_conn))."""
    from oracle import sampler as osamp
    g = golden("hamiltonian_rule_pauli")
    prop, corr = osamp.pauli_hamiltonian_propose(list(g["ops"]), g["weights"], g["x"], g["u"])
    np.testing.assert_array_equal(prop, g["proposed"])
    np.testing.assert_allclose(corr, g["corr"], rtol=0, atol=1e-14)


def test_online_stats_any_chunking_equals_one_shot():
    """For any data and any chunking the accumulated sums equal the one-shot
    ones: the rolling lag buffer pairs samples across chunk boundaries exactly
    (the invariance the reference's tests check for a few chunkings,
    test/stats/test_online_stats.py:50-70, 408-423)."""
    hyp = pytest.importorskip("hypothesis")
    st = pytest.importorskip("hypothesis.strategies")
    from oracle import online_stats as oos

    @hyp.settings(max_examples=60, deadline=None, derandomize=True, database=None)
    @hyp.given(C=st.integers(1, 5), T=st.integers(1, 90), L=st.integers(0, 40),
               seed=st.integers(0, 2 ** 31 - 1), data=st.data())
    def check(C, T, L, seed, data):
        x = np.random.default_rng(seed).normal(size=(C, T)) * 3.0 + 1.0
        cuts = sorted(data.draw(st.sets(st.integers(1, max(1, T - 1)), max_size=8))) if T > 1 \
            else []
        one = oos.update(oos.new_state(C, L), x)
        s = oos.new_state(C, L)
        for ch in np.split(x, cuts, axis=1):
            if ch.shape[1]:
                s = oos.update(s, ch)
        for k in ("count", "cross", "m1", "m2", "pair", "buf"):
            np.testing.assert_allclose(s[k], one[k], rtol=1e-12, atol=1e-10)
        np.testing.assert_allclose(s["mean"], one["mean"], rtol=1e-12, atol=1e-12)
        np.testing.assert_allclose(s["M2"], one["M2"], rtol=1e-9, atol=1e-9)
        assert s["buf_len"] == one["buf_len"] == min(T, L)

    check()
