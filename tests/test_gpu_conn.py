"""Connected elements on the GPU: bit-exact against the oracle (and through it
against the reference's numba kernels), at small sizes element by element and
at the 10x10 J1-J2 size through exact per-element properties."""
import numpy as np
import pytest
import torch

from gpu_common import oracle_heisenberg, oracle_local
from oracle import hilbert as oh
from oracle import operator as oop

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def nk():
    import netket_gb300
    netket_gb300._native.require_cuda()
    return netket_gb300


@pytest.mark.parametrize("name", ["chain16", "chain5", "square4"])
def test_ising_matches_reference_numba(nk, golden, name):
    gi = golden("ising")
    e = golden("edges")[name][:, :2]
    h, J = gi[name + "__hJ"]
    x = oh.local_indices_to_states(gi[name + "__x_ids"])
    N = x.shape[1]
    op = nk.operator.Ising(nk.hilbert.Spin(0.5, N), e, h=h, J=J)
    xp, mels = op.get_conn_padded(torch.as_tensor(x))
    n, K = mels.shape
    ref_xp = oh.local_indices_to_states(gi[name + "__xp_ids"]).reshape(n, K, N)
    np.testing.assert_array_equal(xp.cpu().numpy(), ref_xp)
    np.testing.assert_array_equal(mels.cpu().numpy(), gi[name + "__mels"].reshape(n, K))


@pytest.mark.parametrize("N,h,J", [(16, 1.0, 1.0), (7, 0.3, -2.5), (33, 1.7, 0.25), (12, 0.0, 1.0)])
def test_ising_matches_oracle(nk, N, h, J):
    g = nk.graph.Chain(N)
    op = nk.operator.Ising(nk.hilbert.Spin(0.5, N), g, h=h, J=J)
    x = nk.hilbert.Spin(0.5, N).random_state(seed=N, size=301)
    xp, mels = op.get_conn_padded(x)
    nc = op.n_conn(x)
    rxp, rm = oop.ising_get_conn_padded(x.cpu().numpy(), np.array(g.edges()), h, J)
    np.testing.assert_array_equal(xp.cpu().numpy(), rxp)
    np.testing.assert_array_equal(mels.cpu().numpy(), rm)
    np.testing.assert_array_equal(nc.cpu().numpy(),
                                  oop.ising_n_conn(x.cpu().numpy(), np.array(g.edges()), h, J))


LOCALOP_CASES = ["heis_chain16", "heis_square4", "heis_square4_nosign", "j1j2_square6",
                 "j1j2_chain14", "j1j2_square10", "ising_local_chain5"]


@pytest.mark.parametrize("name", LOCALOP_CASES)
def test_localop_matches_reference_numba(nk, golden, name):
    """Padded output == numba flattened output with |mel| <= 1e-10 dropped (one
    acting-size group) or its lexsorted canonical form (mixed sizes)."""
    gl = golden("localop")
    N = int(gl[name + "__N"])
    ops, aon = [], []
    for a, m, s in zip(gl[name + "__aon"], gl[name + "__ops"], gl[name + "__sizes"]):
        d = 2**int(s)
        ops.append(m[:d, :d])
        aon.append([int(v) for v in a[:s]])
    op = nk.operator.LocalOperator(nk.hilbert.Spin(0.5, N), ops, aon)
    x = oh.local_indices_to_states(gl[name + "__x_ids"])
    xp, mels = op.get_conn_padded(torch.as_tensor(x))
    xp, mels = xp.cpu().numpy(), mels.cpu().numpy()
    nc = op.n_conn(torch.as_tensor(x)).cpu().numpy()
    sections = gl[name + "__sections"]
    ref_xp = oh.local_indices_to_states(gl[name + "__xp_ids"])
    ref_m = gl[name + "__mels"]
    single = len(set(gl[name + "__sizes"].tolist())) == 1
    start = 0
    for b in range(x.shape[0]):
        stop = sections[b]
        keep = np.abs(ref_m[start:stop]) > 1e-10
        rx, rm = ref_xp[start:stop][keep], ref_m[start:stop][keep]
        k = len(rm)
        assert nc[b] == k
        if single:
            np.testing.assert_array_equal(xp[b, :k], rx)
            np.testing.assert_array_equal(mels[b, :k], rm)
        else:
            o1, o2 = np.lexsort(xp[b, :k].T), np.lexsort(rx.T)
            np.testing.assert_array_equal(xp[b, :k][o1], rx[o2])
            np.testing.assert_array_equal(mels[b, :k][o1], rm[o2])
        assert np.all(mels[b, k:] == 0) and np.all(xp[b, k:] == x[b])
        start = stop
    # and the full padded output equals the oracle's JAX-order restatement
    rxp, rm = oracle_local(op).get_conn_padded(x)
    np.testing.assert_array_equal(xp, rxp)
    np.testing.assert_array_equal(mels, rm)


@pytest.mark.parametrize("L,J,order,tsz", [(4, 1.0, 1, 0), (4, [1.0, 0.5], 2, 0), (6, [1.0, 0.5], 2, None),
                                            (3, 1.0, 1, None)])
def test_heisenberg_matches_oracle(nk, L, J, order, tsz):
    g = nk.graph.Square(L, max_neighbor_order=order)
    hi = nk.hilbert.Spin(0.5, N=L * L, total_sz=tsz)
    op = nk.operator.Heisenberg(hi, g, J=J)
    ref = oracle_heisenberg(g, J)
    assert op.max_conn_size == ref.max_conn_size
    x = hi.random_state(seed=11, size=257)
    xp, mels = op.get_conn_padded(x)
    rxp, rm = ref.get_conn_padded(x.cpu().numpy())
    np.testing.assert_array_equal(xp.cpu().numpy(), rxp)
    np.testing.assert_array_equal(mels.cpu().numpy(), rm)


def test_zero_diagonal_is_dropped(nk):
    """States whose diagonal sums to exactly 0 lose the diagonal entry, as in
    the reference's mel_cutoff compaction."""
    g = nk.graph.Chain(4)
    hi = nk.hilbert.Spin(0.5, 4)
    op = nk.operator.Heisenberg(hi, g)
    x = torch.tensor([[1, 1, -1, -1]], dtype=torch.int8)  # two parallel, two antiparallel bonds
    xp, mels = op.get_conn_padded(x)
    rxp, rm = oracle_heisenberg(g).get_conn_padded(x.numpy())
    np.testing.assert_array_equal(mels.cpu().numpy(), rm)
    np.testing.assert_array_equal(xp.cpu().numpy(), rxp)
    assert rm[0, 0] != 0 and not np.any((rxp[0] == x.numpy()[0]).all(axis=1) & (rm[0] != 0))


def test_j1j2_10x10_full_size_properties(nk):
    """16384 samples of the 10x10 J1-J2 model: every kept element is a swap of
    one antiparallel bond with mel 2 J_b, the diagonal equals sum_b J_b x_u x_v,
    padding is (x, 0), and 512 of the samples match the oracle bit for bit."""
    g = nk.graph.Square(10, max_neighbor_order=2)
    hi = nk.hilbert.Spin(0.5, N=100, total_sz=0)
    op = nk.operator.Heisenberg(hi, g, J=[1.0, 0.5])
    assert op.max_conn_size == 401
    x = hi.random_state(seed=5, size=16384)
    xp, mels = op.get_conn_padded(x)
    nc = op.n_conn(x)
    e = np.array(g.edges(return_color=True))
    Jb = np.where(e[:, 2] == 0, 1.0, 0.5)
    xd = x.to(torch.float64)
    prod = xd[:, e[:, 0]] * xd[:, e[:, 1]]
    diag = (prod * torch.as_tensor(Jb, device=x.device)).sum(1)
    n_anti = (prod < 0).sum(1)
    has_diag = diag != 0
    torch.testing.assert_close(nc.to(torch.int64), n_anti + has_diag.to(torch.int64), rtol=0, atol=0)
    d0 = torch.where(has_diag, mels[:, 0], torch.zeros_like(diag))
    torch.testing.assert_close(d0, torch.where(has_diag, diag, torch.zeros_like(diag)), rtol=0, atol=0)
    changed = (xp != x[:, None, :]).sum(-1)
    kidx = torch.arange(401, device=x.device)[None, :]
    kept = kidx < nc[:, None]
    off = kept & ~((kidx == 0) & has_diag[:, None])
    assert torch.all(changed[off] == 2)
    assert torch.all(changed[~kept] == 0) and torch.all(mels[~kept] == 0)
    assert torch.all(xp.to(torch.int32).sum(-1) == 0)  # Sz conserved
    assert torch.all((mels[off] == 2.0) | (mels[off] == 1.0))
    ref = oracle_heisenberg(g, [1.0, 0.5])
    rxp, rm = ref.get_conn_padded(x[:512].cpu().numpy())
    np.testing.assert_array_equal(xp[:512].cpu().numpy(), rxp)
    np.testing.assert_array_equal(mels[:512].cpu().numpy(), rm)


def test_to_sparse_matches_oracle(nk):
    g = nk.graph.Chain(8)
    hi = nk.hilbert.Spin(0.5, 8)
    H = nk.operator.Ising(hi, g, h=0.7)
    A = H.to_dense()
    states = oh.all_states(8)
    ref = oop.to_sparse_from_conn(lambda s: oop.ising_get_conn_padded(s, np.array(g.edges()), 0.7, 1.0),
                                  states).toarray()
    np.testing.assert_array_equal(A, ref)


def test_random_states_match_philox_reference(nk):
    from philox_ref import random_states_ref
    hi = nk.hilbert.Spin(0.5, N=37)
    x = hi.random_state(seed=0x1234567890ABCDEF, size=9, stream_id=3).cpu().numpy()
    np.testing.assert_array_equal(x, random_states_ref(9, 37, -1, 0x1234567890ABCDEF, 3))
    hz = nk.hilbert.Spin(0.5, N=20, total_sz=0)
    xz = hz.random_state(seed=77, size=9, stream_id=1).cpu().numpy()
    np.testing.assert_array_equal(xz, random_states_ref(9, 20, 10, 77, 1))
    big = hz.random_state(seed=1, size=20000).cpu().numpy()
    assert np.all(big.astype(int).sum(1) == 0)
    # every site is down with probability 1/2
    assert np.all(np.abs((big < 0).mean(0) - 0.5) < 0.02)
