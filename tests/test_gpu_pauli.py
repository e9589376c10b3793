"""PauliStrings on the GPU: get_conn_padded / n_conn bit-exact against the
reference's own PauliStringsJax kernel (golden vectors) and the oracle;
fused RBM local energies 1e-10 (FP64) / 1e-4 (FP32) relative against the
oracle and against the dense get_conn + logpsi path."""
import numpy as np
import pytest
import torch

from gpu_common import oracle_params
from oracle import hilbert as oh
from oracle import operator as oop
from oracle import rbm as orbm

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def nk():
    import netket_gb300
    netket_gb300._native.require_cuda()
    return netket_gb300


def random_strings(rng, N, n, max_len):
    ops, w = [], []
    for _ in range(n):
        s = ["I"] * N
        k = int(rng.integers(1, max_len + 1))
        for i in rng.choice(N, size=k, replace=False):
            s[i] = "XYZ"[int(rng.integers(0, 3))]
        if s.count("Y") % 2:
            i = s.index("Y")
            s[i] = "X"
        ops.append("".join(s))
        w.append(float(rng.normal()))
    # repeat some flip sets with other Z / weights so that slots hold several strings
    for o in list(ops[: n // 4]):
        ops.append(o.replace("Z", "I"))
        w.append(float(rng.normal()))
    return ops, w


@pytest.mark.parametrize("name", ["tfim", "heisenberg_xyz", "mixed", "duplicates_and_zeros"])
def test_pauli_conn_matches_reference(nk, golden, name):
    """From the raw strings through the constructor's reduction."""
    g = golden("pauli_strings")
    ops, w = list(g[name + "__raw_ops"]), g[name + "__raw_weights"]
    N = len(ops[0])
    op = nk.operator.PauliStrings(nk.hilbert.Spin(0.5, N), ops, w)
    x = torch.as_tensor(oh.local_indices_to_states(g[name + "__x_ids"]), device="cuda")
    xp, mels = op.get_conn_padded(x)
    np.testing.assert_array_equal(xp.cpu().numpy(),
                                  oh.local_indices_to_states(g[name + "__xp_ids"]))
    np.testing.assert_array_equal(mels.cpu().numpy(), g[name + "__mels"])
    np.testing.assert_array_equal(op.n_conn(x).cpu().numpy(), g[name + "__n_conn"])


@pytest.mark.parametrize("N,n_str,max_len", [(40, 60, 6), (100, 150, 12), (33, 20, 33)])
def test_pauli_conn_matches_oracle(nk, N, n_str, max_len):
    rng = np.random.default_rng(N)
    ops, w = random_strings(rng, N, n_str, max_len)
    op = nk.operator.PauliStrings(nk.hilbert.Spin(0.5, N), ops, w)
    x = nk.hilbert.Spin(0.5, N).random_state(seed=N, size=97)
    xp, mels = op.get_conn_padded(x)
    rxp, rm, rn = oop.pauli_get_conn_padded(x.cpu().numpy(), ops, w)
    np.testing.assert_array_equal(xp.cpu().numpy(), rxp)
    np.testing.assert_allclose(mels.cpu().numpy(), rm, rtol=1e-15, atol=0)
    np.testing.assert_array_equal(op.n_conn(x).cpu().numpy(), rn)


@pytest.mark.parametrize("dtype,rtol", [(torch.float64, 1e-10), (torch.float32, 1e-4)])
@pytest.mark.parametrize("N,alpha", [(40, 1), (100, 2)])
def test_pauli_eloc_fused(nk, dtype, rtol, N, alpha):
    rng = np.random.default_rng(N + alpha)
    ops, w = random_strings(rng, N, 2 * N, 8)
    hi = nk.hilbert.Spin(0.5, N)
    op = nk.operator.PauliStrings(hi, ops, w)
    model = nk.models.RBM(alpha=alpha, kernel_init_std=0.05, hidden_bias_init_std=0.05,
                          visible_bias_init_std=0.05)
    flat = model.init_flat(3, N)
    M = model.n_hidden(N)
    x = hi.random_state(seed=7, size=300)
    e = nk.kernels.local_energies_fused(op, flat.to(dtype), x, N, M)
    p = oracle_params(flat, N, M)
    ref = orbm.local_energies(p, x.cpu().numpy(),
                              lambda xx: oop.pauli_get_conn_padded(xx, ops, w)[:2])
    scale = np.abs(ref).max()
    np.testing.assert_allclose(e.cpu().numpy(), ref, rtol=0, atol=rtol * scale)
    if dtype == torch.float64:
        ed = nk.kernels.local_energies_dense(op, flat, x, N, M)
        np.testing.assert_allclose(e.cpu().numpy(), ed.cpu().numpy(), rtol=0, atol=1e-12 * scale)


def test_pauli_tfim_equals_ising(nk):
    """The transverse-field Ising model written as Pauli strings gives the
    Ising operator's local energies."""
    N = 24
    hi = nk.hilbert.Spin(0.5, N)
    gr = nk.graph.Chain(N)
    ising = nk.operator.Ising(hi, gr, h=0.7, J=1.3)
    ops = ["".join("X" if k == i else "I" for k in range(N)) for i in range(N)]
    ops += ["".join("Z" if k in (i, j) else "I" for k in range(N)) for i, j in gr.edges()]
    op = nk.operator.PauliStrings(hi, ops, [-0.7] * N + [1.3] * len(gr.edges()))
    assert op.max_conn_size == N + 1
    model = nk.models.RBM(alpha=2)
    flat = model.init_flat(5, N)
    x = hi.random_state(seed=2, size=500)
    a = nk.kernels.local_energies_fused(op, flat, x, N, model.n_hidden(N))
    b = nk.kernels.local_energies_fused(ising, flat, x, N, model.n_hidden(N))
    torch.testing.assert_close(a, b, rtol=1e-12, atol=1e-12)
