"""Statistics, Jacobian contractions, Gram matrices, solvers and the SR /
minSR updates on the GPU against the oracle (FP64: 1e-10 relative)."""
import math

import numpy as np
import pytest
import torch

from gpu_common import oracle_heisenberg, oracle_params
from oracle import ngd as ongd
from oracle import rbm as orbm
from oracle import stats as ost

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def nk():
    import netket_gb300
    netket_gb300._native.require_cuda()
    return netket_gb300


@pytest.mark.parametrize("name", ["c1", "c2", "odd", "onechain", "wide", "ar1_blocks", "ar1_slow"])
def test_stats_match_reference(nk, golden, name):
    g = golden("stats")
    s = nk.stats.statistics(g[name + "__data"]).as_array()
    np.testing.assert_allclose(s, g[name + "__stats"], rtol=1e-11, atol=1e-13, equal_nan=True)


def test_stats_large_matches_oracle(nk):
    rng = np.random.default_rng(0)
    d = rng.normal(-3, 2, size=(4096, 4)) + rng.normal(size=(4096, 1))
    np.testing.assert_allclose(nk.stats.statistics(d).as_array(), ost.statistics(d).as_array(),
                               rtol=1e-11, equal_nan=True)


def _problem(nk, N, M_alpha, n, seed=0, std=0.2):
    model = nk.models.RBM(alpha=M_alpha, kernel_init_std=std, hidden_bias_init_std=std,
                          visible_bias_init_std=std)
    flat = model.init_flat(seed, N)
    M = model.n_hidden(N)
    x = nk.hilbert.Spin(0.5, N).random_state(seed=seed + 1, size=n)
    _, _, t = nk.kernels.rbm_forward(flat, x, N, M, want_tanh=True)
    p = oracle_params(flat, N, M)
    return model, flat, M, x, t, p


@pytest.mark.parametrize("N,alpha,n", [(16, 1, 1008), (30, 3, 2500), (100, 4, 1200)])
def test_ot_v_and_jacobian(nk, N, alpha, n):
    model, flat, M, x, t, p = _problem(nk, N, alpha, n)
    rng = np.random.default_rng(1)
    v = rng.normal(size=n)
    got = nk.kernels.ot_v(t, x, N, M, torch.as_tensor(v, device=x.device)).cpu().numpy()
    O = orbm.jacobian(p, x.cpu().numpy())
    np.testing.assert_allclose(got, O.T @ v, rtol=1e-10, atol=1e-10 * np.abs(O.T @ v).max())
    t32 = t.float()
    got32 = nk.kernels.ot_v(t32, x, N, M, torch.as_tensor(v, device=x.device)).cpu().numpy()
    np.testing.assert_allclose(got32, O.T @ v, rtol=1e-4, atol=1e-5 * np.abs(O.T @ v).max() + 1e-5)
    obar = nk.kernels.column_means(t, x, N, M)
    OL = nk.kernels.jacobian_dense(t, x, N, M, obar, 1 / math.sqrt(n), torch.float64)
    ref = (O - O.mean(0)) / math.sqrt(n)
    np.testing.assert_allclose(OL.cpu().numpy(), ref, rtol=1e-10, atol=1e-12)


@pytest.mark.parametrize("N,alpha,n", [(16, 1, 500), (36, 2, 700), (100, 4, 400)])
def test_structured_gram(nk, N, alpha, n):
    model, flat, M, x, t, p = _problem(nk, N, alpha, n)
    O = orbm.jacobian(p, x.cpu().numpy(), center=True) / math.sqrt(n)
    ref = O @ O.T + 1e-3 * np.eye(n)
    low = np.tril_indices(n)
    obar = nk.kernels.column_means(t, x, N, M)
    T64, _ = nk.kernels.gram_structured(t, x, N, M, obar, 1e-3, mode=0)
    np.testing.assert_allclose(T64.cpu().numpy()[low], ref[low], rtol=1e-10,
                               atol=1e-12 * np.abs(ref).max())
    T64b, T32 = nk.kernels.gram_structured(t.float(), x, N, M, obar, 1e-3, mode=1, want_f32=True)
    np.testing.assert_allclose(T64b.cpu().numpy()[low], ref[low], rtol=1e-4,
                               atol=1e-5 * np.abs(ref).max())
    np.testing.assert_allclose(T32.cpu().numpy()[low], ref[low], rtol=1e-4,
                               atol=1e-5 * np.abs(ref).max())
    OL = nk.kernels.jacobian_dense(t, x, N, M, obar, 1 / math.sqrt(n), torch.float64)
    Td = nk.kernels.gram_dense(OL, 1e-3)
    np.testing.assert_allclose(Td.cpu().numpy()[low], ref[low], rtol=1e-10,
                               atol=1e-12 * np.abs(ref).max())
    S = nk.kernels.gram_dense(OL, 1e-3, transpose=True)
    P = O.shape[1]
    refS = O.T @ O + 1e-3 * np.eye(P)
    lowP = np.tril_indices(P)
    np.testing.assert_allclose(S.cpu().numpy()[lowP], refS[lowP], rtol=1e-10,
                               atol=1e-12 * np.abs(refS).max())


def test_solvers(nk, golden):
    g = golden("ngd")
    A = torch.as_tensor(g["solve_spd__A"], device="cuda")
    b = torch.as_tensor(g["solve_spd__b"], device="cuda")
    x, info = nk.ngd.solve_with_fallback(A, b)
    np.testing.assert_allclose(x.cpu().numpy(), g["solve_spd__x"], rtol=1e-10)
    assert not info["solver_fallback"]
    An = A.clone()
    An[0, 0] = float("nan")
    _, info = nk.ngd.solve_with_fallback(An, b)
    assert info["solver_fallback"] and bool(g["solve_nan__fallback"])
    S = torch.as_tensor(g["pinv_singular__A"], device="cuda")
    xs = nk.kernels.pinv_smooth_solve(S, torch.as_tensor(g["pinv_singular__b"], device="cuda"))
    np.testing.assert_allclose(xs.cpu().numpy(), g["pinv_singular__x"], rtol=1e-8, atol=1e-10)
    # singular (rank-deficient) matrix without shift: Cholesky fails -> pinv fallback
    x2, info2 = nk.ngd.solve_with_fallback(S, torch.as_tensor(g["pinv_singular__b"], device="cuda"))
    assert info2["solver_fallback"]


def test_refined_solve(nk):
    rng = np.random.default_rng(3)
    n = 700
    U = rng.normal(size=(n, 200))
    A = U @ U.T / 200 + 1e-3 * np.eye(n)
    b = rng.normal(size=n)
    At = torch.as_tensor(A, device="cuda")
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    x, res = nk.kernels.cholesky_solve_refined(At, At.float().contiguous(), torch.as_tensor(b, device="cuda"),
                                               st, max_iter=6, tol=1e-12)
    np.testing.assert_allclose(x.cpu().numpy(), np.linalg.solve(A, b), rtol=1e-9,
                               atol=1e-9 * np.abs(np.linalg.solve(A, b)).max())
    assert res.item() < 1e-12 and st.item() == 0


@pytest.mark.parametrize("name", ["minsr", "sr", "minsr_big_shift"])
def test_dense_solve_path_matches_reference_ngd(nk, golden, name):
    """The dense QGT / NTK solves of the reference on its own random inputs."""
    g = golden("ngd")
    O, e, shift = g[name + "__O"], g[name + "__e"], float(g[name + "__shift"])
    n = O.shape[0]
    O_L = torch.as_tensor(O / math.sqrt(n), device="cuda")
    dv = torch.as_tensor(2 * (e - e.mean()) / math.sqrt(n), device="cuda")
    if name.startswith("minsr"):
        T = nk.kernels.gram_dense(O_L, shift)
        aux, _ = nk.ngd.solve_with_fallback(T, dv)
        upd = (O_L.T @ aux).cpu().numpy()
    else:
        S = nk.kernels.gram_dense(O_L, shift, transpose=True)
        upd, _ = nk.ngd.solve_with_fallback(S, O_L.T @ dv)
        upd = upd.cpu().numpy()
    np.testing.assert_allclose(upd, g[name + "__update"], rtol=1e-9, atol=1e-11)


@pytest.mark.parametrize("gram,solve", [("structured", "cholesky"), ("dense", "cholesky"),
                                        ("structured", "refined")])
def test_minsr_update_matches_oracle(nk, gram, solve):
    N, n = 16, 512
    model, flat, M, x, t, p = _problem(nk, N, 2, n, seed=4)
    g = nk.graph.Chain(N)
    H = nk.operator.Heisenberg(nk.hilbert.Spin(0.5, N), g)
    e = nk.kernels.local_energies_fused(H, flat, x, N, M)
    mean = e.mean().reshape(1)
    t_in = t if solve != "refined" else t.float()
    dp, info = nk.ngd.minsr_update(t_in, x, N, M, e, mean, 1e-4, gram=gram, solve=solve,
                                   refine_iters=8, refine_tol=1e-9)
    O = orbm.jacobian(p, x.cpu().numpy(), center=True)
    ref, _ = ongd.srt_update(O, e.cpu().numpy(), 1e-4)
    tol = 1e-8 if solve != "refined" else 2e-3
    np.testing.assert_allclose(dp.cpu().numpy(), ref, rtol=tol, atol=tol * np.abs(ref).max())
    assert not info["solver_fallback"]


def test_sr_equals_minsr(nk):
    """Woodbury identity on the device (test/driver/test_srt.py:98-175, atol 1e-10)."""
    N, n = 8, 96
    model, flat, M, x, t, p = _problem(nk, N, 1, n, seed=6)
    e = torch.as_tensor(np.random.default_rng(0).normal(size=n), device="cuda")
    mean = e.mean().reshape(1)
    a, _ = nk.ngd.minsr_update(t, x, N, M, e, mean, 1e-3)
    b, _ = nk.ngd.sr_update(t, x, N, M, e, mean, 1e-3)
    np.testing.assert_allclose(a.cpu().numpy(), b.cpu().numpy(), atol=1e-10)
