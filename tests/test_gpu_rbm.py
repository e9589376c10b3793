"""RBM log-amplitudes and local energies on the GPU against the FP64 oracle.
Tolerances: FP64 kernels 1e-10 relative (the accuracy stated for FP64 paths);
FP32 kernels 2e-5 relative on log-amplitudes and 1e-4 on local energies."""
import numpy as np
import pytest
import torch

from gpu_common import oracle_heisenberg, oracle_params
from oracle import operator as oop
from oracle import rbm as orbm

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def nk():
    import netket_gb300
    netket_gb300._native.require_cuda()
    return netket_gb300


def _setup(nk, N, alpha, seed, std=0.1):
    model = nk.models.RBM(alpha=alpha, kernel_init_std=std, hidden_bias_init_std=std,
                          visible_bias_init_std=std)
    flat = model.init_flat(seed, N)
    return model, flat, model.n_hidden(N)


@pytest.mark.parametrize("N,alpha", [(16, 1), (100, 4), (37, 2), (256, 1)])
def test_logpsi(nk, N, alpha):
    model, flat, M = _setup(nk, N, alpha, N)
    x = nk.hilbert.Spin(0.5, N).random_state(seed=1, size=1000)
    lp64 = model.apply(flat, x, dtype=torch.float64).cpu().numpy()
    lp32 = model.apply(flat, x, dtype=torch.float32).cpu().numpy()
    ref = orbm.logpsi(oracle_params(flat, N, M), x.cpu().numpy())
    np.testing.assert_allclose(lp64, ref, rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(lp32, ref, rtol=2e-5, atol=2e-5)
    _, th, tt = nk.kernels.rbm_forward(flat, x, N, M, want_theta=True, want_tanh=True)
    rth = orbm.theta(oracle_params(flat, N, M), x.cpu().numpy())
    np.testing.assert_allclose(th.cpu().numpy(), rth, rtol=1e-12, atol=1e-13)
    np.testing.assert_allclose(tt.cpu().numpy(), np.tanh(rth), rtol=1e-12, atol=1e-13)


TC_CASES = [(100, 4, 3000), (256, 8, 1500), (37, 3, 777)]


@pytest.mark.parametrize("N,alpha,n", TC_CASES)
def test_logpsi_tensor_cores(nk, N, alpha, n):
    """theta = x W on tcgen05 (W split into FP16 hi + lo, x exact) for FP32
    parameters: the 10x10 alpha-4 and 16x16 alpha-8 widths and an odd N (site
    padding) with n not a multiple of the tile: logpsi, theta and tanh theta
    against the FP64 oracle of the same FP32 parameters (FP32 tolerances) and
    against the CUDA-core FP32 kernel."""
    model, flat, M = _setup(nk, N, alpha, N + 3)
    f32 = flat.float()
    x = nk.hilbert.Spin(0.5, N).random_state(seed=2, size=n)
    lp, th, tt = nk.kernels.rbm_forward(f32, x, N, M, want_theta=True, want_tanh=True,
                                        use_tc=True)
    p = oracle_params(f32.double(), N, M)
    xs = x.cpu().numpy()
    rth = orbm.theta(p, xs)
    np.testing.assert_allclose(th.cpu().numpy(), rth, rtol=1e-5, atol=2e-5)
    np.testing.assert_allclose(tt.cpu().numpy(), np.tanh(rth), rtol=1e-5, atol=2e-5)
    np.testing.assert_allclose(lp.cpu().numpy(), orbm.logpsi(p, xs), rtol=2e-5, atol=2e-5)
    lp_c, _, _ = nk.kernels.rbm_forward(f32, x, N, M, use_tc=False)
    np.testing.assert_allclose(lp.cpu().numpy(), lp_c.cpu().numpy(), rtol=2e-5, atol=2e-5)
    # without a theta buffer the pre-activation lives in the workspace
    lp2, _, tt2 = nk.kernels.rbm_forward(f32, x, N, M, want_tanh=True, use_tc=True)
    assert torch.equal(lp2, lp) and torch.equal(tt2, tt)


@pytest.mark.parametrize("N,alpha,n", TC_CASES)
def test_ot_v_tensor_cores(nk, N, alpha, n):
    """O^T v on tcgen05 (v t split into FP16 hi + lo, samples split into K
    chunks, partial sums in FP64): the kernel, hidden-bias and visible-bias parts
    against the FP64 product with the same FP32 t, and against the CUDA-core
    FP32 kernel (FP32 tolerances, 1e-4 relative)."""
    model, flat, M = _setup(nk, N, alpha, N + 5)
    f32 = flat.float()
    x = nk.hilbert.Spin(0.5, N).random_state(seed=3, size=n)
    _, _, t = nk.kernels.rbm_forward(f32, x, N, M, want_tanh=True, use_tc=False)
    v = torch.as_tensor(np.random.default_rng(n).normal(size=n), device="cuda")
    got = nk.kernels.ot_v(t, x, N, M, v, use_tc=True).cpu().numpy()
    tn = t.double().cpu().numpy()
    xs = x.cpu().numpy().astype(np.float64)
    O = np.concatenate([tn, (xs[:, :, None] * tn[:, None, :]).reshape(n, N * M), xs], axis=1)
    ref = O.T @ v.cpu().numpy()
    scale = np.abs(ref).max()
    np.testing.assert_allclose(got, ref, rtol=1e-4, atol=1e-5 * scale)
    simt = nk.kernels.ot_v(t, x, N, M, v, use_tc=False).cpu().numpy()
    np.testing.assert_allclose(got, simt, rtol=1e-4, atol=1e-5 * scale)


@pytest.mark.parametrize("N,h,J", [(16, 1.0, 1.0), (24, 0.6, -1.0), (9, 0.0, 1.0)])
def test_eloc_ising(nk, N, h, J):
    model, flat, M = _setup(nk, N, 2, 3)
    g = nk.graph.Chain(N)
    H = nk.operator.Ising(nk.hilbert.Spin(0.5, N), g, h=h, J=J)
    x = nk.hilbert.Spin(0.5, N).random_state(seed=2, size=777)
    p = oracle_params(flat, N, M)
    ref = orbm.local_energies(p, x.cpu().numpy(),
                              lambda s: oop.ising_get_conn_padded(s, np.array(g.edges()), h, J))
    e64 = nk.kernels.local_energies_fused(H, flat, x, N, M).cpu().numpy()
    d64 = nk.kernels.local_energies_dense(H, flat, x, N, M).cpu().numpy()
    e32 = nk.kernels.local_energies_fused(H, flat.float(), x, N, M).cpu().numpy()
    d32 = nk.kernels.local_energies_dense(H, flat.float(), x, N, M).cpu().numpy()
    np.testing.assert_allclose(e64, ref, rtol=1e-10, atol=1e-10)
    np.testing.assert_allclose(d64, ref, rtol=1e-10, atol=1e-10)
    scale = np.abs(ref).max()
    np.testing.assert_allclose(e32, ref, rtol=1e-4, atol=1e-4 * scale)
    np.testing.assert_allclose(d32, ref, rtol=1e-4, atol=1e-4 * scale)


@pytest.mark.parametrize("L,J,order,alpha,sign_rule", [
    (4, 1.0, 1, 2, None), (6, [1.0, 0.5], 2, 2, None), (10, [1.0, 0.5], 2, 2, None),
    # the benchmark's Hamiltonian and width: 10x10 J1-J2, Marshall sign on J1, M = 400
    (10, [1.0, 0.5], 2, 4, [True, False])])
def test_eloc_heisenberg(nk, L, J, order, alpha, sign_rule):
    N = L * L
    model, flat, M = _setup(nk, N, alpha, 4)
    g = nk.graph.Square(L, max_neighbor_order=order)
    hi = nk.hilbert.Spin(0.5, N, total_sz=0)
    H = nk.operator.Heisenberg(hi, g, J=J, sign_rule=sign_rule)
    x = hi.random_state(seed=9, size=300)
    ref = orbm.local_energies(oracle_params(flat, N, M), x.cpu().numpy(),
                              oracle_heisenberg(g, J, sign_rule).get_conn_padded)
    e64 = nk.kernels.local_energies_fused(H, flat, x, N, M).cpu().numpy()
    d64 = nk.kernels.local_energies_dense(H, flat, x, N, M).cpu().numpy()
    e32 = nk.kernels.local_energies_fused(H, flat.float(), x, N, M).cpu().numpy()
    np.testing.assert_allclose(e64, ref, rtol=1e-10, atol=1e-10)
    np.testing.assert_allclose(d64, ref, rtol=1e-10, atol=1e-10)
    np.testing.assert_allclose(e32, ref, rtol=1e-4, atol=1e-4 * np.abs(ref).max())


def test_eloc_general_local_operator(nk):
    """1-site and 2-site terms together (Ising written as a LocalOperator) plus
    a constant: fused == dense == oracle."""
    N = 10
    model, flat, M = _setup(nk, N, 1, 5)
    hi = nk.hilbert.Spin(0.5, N)
    H = nk.operator.Ising(hi, nk.graph.Chain(N), h=0.8, J=1.1).to_local_operator() + 0.25
    x = hi.random_state(seed=4, size=200)
    ref_op = oop.LocalOperator(N, H.operators, H.acting_on, constant=0.25)
    ref = orbm.local_energies(oracle_params(flat, N, M), x.cpu().numpy(), ref_op.get_conn_padded)
    e = nk.kernels.local_energies_fused(H, flat, x, N, M).cpu().numpy()
    d = nk.kernels.local_energies_dense(H, flat, x, N, M).cpu().numpy()
    np.testing.assert_allclose(e, ref, rtol=1e-10, atol=1e-10)
    np.testing.assert_allclose(d, ref, rtol=1e-10, atol=1e-10)
