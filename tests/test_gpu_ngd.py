"""Statistics, Jacobian contractions, Gram matrices, solvers and the SR /
minSR updates on the GPU against the oracle (FP64: 1e-10 relative)."""
import math

import numpy as np
import pytest
import torch

from gpu_common import oracle_params
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


def _jacobian_from_t(t, x):
    n, N = x.shape
    M = t.shape[1]
    return np.concatenate([t, (x[:, :, None] * t[:, None, :]).reshape(n, N * M), x], axis=1)


def _round_terms(v, terms):
    if terms == 0:
        return v
    if terms == 3:  # mode 4: the 2^-19 fixed-point grid
        return torch.round(v * 524288.0) / 524288.0
    hi = v.to(torch.bfloat16).float()
    return hi if terms == 1 else hi + (v - hi).to(torch.bfloat16).float()


@pytest.mark.parametrize("N,alpha,n", [(16, 1, 300), (100, 4, 700), (36, 2, 1030)])
def test_fp32_and_tensor_core_gram(nk, N, alpha, n):
    """FP32 Gram modes contract c = round(t - s0) (s0 = fp32 column mean of t;
    mode 1 FP32, mode 2 hi + lo BF16 pairs on tcgen05, mode 3 one BF16 on
    tcgen05, mode 4 rounded to 2^-19 and split into fixed-point FP16 hi + lo
    whose slab sums are exact) and add the shift back exactly: T equals the FP64 Gram of the
    Jacobian of t_eff = c + s0 centred at the given obar, to FP32 accumulation
    accuracy, and is positive definite."""
    model, flat, M, x, t, p = _problem(nk, N, alpha, n)
    xs = x.cpu().numpy().astype(np.float64)
    low = np.tril_indices(n)
    t32 = t.float().contiguous()
    obar = nk.kernels.column_means(t, x, N, M)
    s0 = obar[:M].float()
    ob = obar.cpu().numpy()
    for mode, terms in ((1, 0), (2, 2), (3, 1), (4, 3)):
        teff = (_round_terms(t32 - s0, terms).double() + s0.double()).cpu().numpy()
        O = (_jacobian_from_t(teff, xs) - ob) / math.sqrt(n)
        ref = O @ O.T + 1e-3 * np.eye(n)
        scale = np.abs(ref).max()
        st = torch.zeros(1, dtype=torch.int32, device="cuda")
        T64, T32 = nk.kernels.gram_structured(t32, x, N, M, obar, 1e-3, mode=mode, want_f32=True,
                                              status=st)
        assert st.item() == 0
        got = T64.cpu().numpy()
        err = np.abs(got[low] - ref[low]).max() / scale
        assert err < 2e-6, (mode, err)
        np.testing.assert_allclose(T32.cpu().numpy()[low], got[low], rtol=1e-6, atol=1e-7 * scale)
        full = np.tril(got) + np.tril(got, -1).T
        np.linalg.cholesky(full)  # positive definite


def _structured_gram_f64(teff, xs, ob, n, shift):
    """O_L O_L^T + shift I in FP64 from the identity O(s).O(s') =
    (t_s.t_s')(1 + x_s.x_s') + x_s.x_s' and g = O obar, without forming O."""
    N, M = xs.shape[1], teff.shape[1]
    X = xs @ xs.T
    G = (teff @ teff.T) * (1.0 + X) + X
    Wb = ob[M:M + N * M].reshape(N, M)
    g = teff @ ob[:M] + np.einsum("si,ij,sj->s", xs, Wb, teff) + xs @ ob[M + N * M:]
    return (G - g[:, None] - g[None, :] + ob @ ob) / n + shift * np.eye(n)


@pytest.mark.parametrize("N,alpha,n", [(256, 8, 2048), (64, 10, 1500), (256, 8, 8192)])
def test_tensor_core_gram_large_m(nk, N, alpha, n):
    """M > 512 (the 16 x 16, alpha 8 model's M = 2048): the default mode 4 Gram
    equals the FP64 Gram of t_eff = c + s0, c = fp32(t - s0) rounded to a
    multiple of 2^-19, to 2e-6 of its largest
    entry and is positive definite at diag_shift 1e-4 with the model's default
    N(0, 0.01) initialisation; it is the mode minsr_update picks there."""
    model, flat, M, x, t, p = _problem(nk, N, alpha, n, std=0.01)
    assert M > nk.ngd.TC_GRAM_MAX_M
    xs = x.cpu().numpy().astype(np.float64)
    low = np.tril_indices(n)
    t32 = t.float().contiguous()
    obar = nk.kernels.column_means(t, x, N, M)
    s0 = obar[:M].float()
    ob = obar.cpu().numpy()
    teff = (_round_terms(t32 - s0, 3).double() + s0.double()).cpu().numpy()
    ref = _structured_gram_f64(teff, xs, ob, n, 1e-4)
    scale = np.abs(ref).max()
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    T64, T32 = nk.kernels.gram_structured(t32, x, N, M, obar, 1e-4, mode=4, want_f32=True,
                                          status=st)
    assert st.item() == 0
    got = T64.cpu().numpy()
    err = np.abs(got[low] - ref[low]).max() / scale
    assert err < 2e-6, err
    np.testing.assert_allclose(T32.cpu().numpy()[low], got[low], rtol=1e-6, atol=1e-7 * scale)
    full = np.tril(got) + np.tril(got, -1).T
    np.linalg.cholesky(full)


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


@pytest.mark.parametrize("n,mode", [(700, 2), (2500, 0), (2500, 1), (2500, 2), (4100, 2),
                                    (100, 3), (700, 3), (1278, 3), (2500, 3), (4100, 3),
                                    (100, 4), (128, 4), (700, 4), (1278, 4), (2500, 4),
                                    (4100, 4), (5000, 4)])
def test_refined_solve(nk, n, mode):
    """FP32-accurate factorisation (cuSOLVER, emulated cuSOLVER, recursive GEMM
    Cholesky, blocked Cholesky with the library's leaf kernel, the library's
    tensor-core Cholesky) + refinement with a double-float residual reaches the
    FP64 solution.  Mode 4 covers a single leaf (100, 128), partial panels and
    block rows (700, 1278: padded to a multiple of 4, 2500, 4100) and several
    512-row block rows (5000)."""
    rng = np.random.default_rng(3)
    U = rng.normal(size=(n, 300))
    A = U @ U.T / 300 + 1e-3 * np.eye(n)
    b = rng.normal(size=n)
    At = torch.as_tensor(A, device="cuda")
    A32 = At.float().contiguous()
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    x, res = nk.kernels.cholesky_solve_refined(At, A32, torch.as_tensor(b, device="cuda"),
                                               st, max_iter=6, tol=1e-10, factor_mode=mode)
    ref = np.linalg.solve(A, b)
    np.testing.assert_allclose(x.cpu().numpy(), ref, rtol=1e-9, atol=1e-9 * np.abs(ref).max())
    # the residual is evaluated in double-float (~2^-46 per term): with cond(A) up to
    # ~2e4 here its floor is ~1e-11 to 3e-11 relative
    assert res.item() < 1e-10 and st.item() == 0
    # the factor itself: U^T U == A to FP32 accuracy (upper triangle, column-major
    # == lower triangle, row-major)
    L = torch.tril(A32).double()
    np.testing.assert_allclose((L @ L.T).cpu().numpy(), A, atol=2e-5 * np.abs(A).max())


_TALL_BLOCKS = r"""
import sys
import numpy as np, torch
sys.path.insert(0, {root!r})
import netket_gb300 as nk
n = {n}
rng = np.random.default_rng(5)
U = rng.normal(size=(n, 300))
A = U @ U.T / 300 + 1e-3 * np.eye(n)
b = rng.normal(size=n)
At = torch.as_tensor(A, device="cuda")
A32 = At.float().contiguous()
st = torch.zeros(1, dtype=torch.int32, device="cuda")
x, res = nk.kernels.cholesky_solve_refined(At, A32, torch.as_tensor(b, device="cuda"), st,
                                           max_iter=6, tol=1e-10)
ref = np.linalg.solve(A, b)
L = torch.tril(A32).double()
print(st.item(), res.item(), np.abs(x.cpu().numpy() - ref).max() / np.abs(ref).max(),
      np.abs((L @ L.T).cpu().numpy() - A).max() / np.abs(A).max())
"""


@pytest.mark.parametrize("blk,n", [(1024, 2600), (1024, 4100), (2048, 4100), (2048, 5000)])
def test_refined_solve_tall_row_blocks(nk, blk, n):
    """The 1024- and 2048-row block rows the factorisation takes from n = 16,384
    and 49,152 on (8 / 16 inner panels per block row, K = 1024 / 2048 trailing
    updates), forced on smaller matrices with partial block rows
    (VMCK_CHOL_BLOCK is read once per process: a child process): the factor
    equals A to FP32 accuracy and the refined solve the FP64 solution."""
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, VMCK_CHOL_BLOCK=str(blk))
    out = subprocess.run([sys.executable, "-c", _TALL_BLOCKS.format(root=root, n=n)], env=env,
                         capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr[-2000:]
    st, res, xerr, ferr = out.stdout.split()[-4:]
    assert int(st) == 0 and float(res) < 1e-10, out.stdout
    assert float(xerr) < 1e-9 and float(ferr) < 2e-5, out.stdout


@pytest.mark.parametrize("mode", [2, 3, 4])
def test_refined_solve_flags_non_spd(nk, mode):
    n = 1500
    A = -np.eye(n)
    At = torch.as_tensor(A, device="cuda")
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    nk.kernels.cholesky_solve_refined(At, At.float().contiguous(), torch.ones(n, device="cuda",
                                      dtype=torch.float64), st, max_iter=2, factor_mode=mode)
    assert st.item() & nk._native.DEV_NOT_SPD


def _ill_conditioned(n, lo, hi, seed):
    rng = np.random.default_rng(seed)
    Q, _ = np.linalg.qr(rng.normal(size=(n, n)))
    d = np.logspace(np.log10(hi), np.log10(lo), n)
    return (Q * d) @ Q.T, rng.normal(size=n)


@pytest.mark.parametrize("n", [1000, 1536])
def test_pcg_solves_beyond_the_fp32_factor(nk, n):
    """cond(A) = 1e8: the FP32 factor (and its refinement) cannot solve A, the
    FP64 Cholesky of the reference can; the shifted-factor PCG reaches an FP64
    residual of 1e-8 ||b|| (FP64's own floor eps ||A|| ||x|| is ~2e-9 ||b||
    here) and the FP64 solution to 1e-6 (n = 1000 also runs the padded factor)."""
    A, b = _ill_conditioned(n, 1e-6, 1e2, seed=n)
    At = torch.as_tensor(np.tril(A), device="cuda")
    bt = torch.as_tensor(b, device="cuda")
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    nk.kernels.cholesky_solve_refined(At, At.float().contiguous(), bt, st, max_iter=8,
                                      tol=1e-8)
    assert st.item() != 0  # the mixed solve does not get there
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    x, res, mu = nk.kernels.cholesky_solve_pcg(At, bt, st, tol=1e-8)
    assert st.item() == 0, (st.item(), res.item(), mu)
    assert mu > 0
    xs = x.cpu().numpy()
    assert np.linalg.norm(A @ xs - b) <= 2e-8 * np.linalg.norm(b)
    assert res.item() <= 1e-8
    ref = np.linalg.solve(A, b)
    assert np.linalg.norm(xs - ref) <= 1e-6 * np.linalg.norm(ref)


def test_minsr_falls_back_to_pcg(nk):
    """Repeated samples (an exactly singular O_L O_L^T) and diag_shift = ||T|| / 1e8:
    the FP32 factor of T fails; minsr_update (refined solve, FP64 T) then solves
    T by shifted-factor PCG -- not pinv_smooth -- to its refine_tol of 1e-7 (the
    FP64 floor eps cond(T) is ~1e-8)."""
    N, n = 16, 512
    model, flat, M, x, t, p = _problem(nk, N, 2, 64, seed=9)
    x = x.repeat(8, 1)
    _, _, t = nk.kernels.rbm_forward(flat, x, N, M, want_tanh=True)
    g = nk.graph.Chain(N)
    H = nk.operator.Heisenberg(nk.hilbert.Spin(0.5, N), g)
    e = nk.kernels.local_energies_fused(H, flat, x, N, M)
    obar = nk.kernels.column_means(t, x, N, M)
    T0, _ = nk.kernels.gram_structured(t, x, N, M, obar, 0.0, 0)
    T0 = torch.tril(T0) + torch.tril(T0, -1).T
    shift = float(torch.linalg.eigvalsh(T0)[-1]) / 1e8
    dp, info = nk.ngd.minsr_update(t, x, N, M, e, e.mean().reshape(1), shift, solve="refined",
                                   refine_tol=1e-7)
    assert info["status"] != 0
    assert info["pcg"]["status"] == 0 and not info["solver_fallback"], info["pcg"]
    T = (T0 + shift * torch.eye(n, dtype=torch.float64, device="cuda")).cpu().numpy()
    dv = (2 * (e - e.mean()) / math.sqrt(n)).cpu().numpy()
    aux = info["aux"].cpu().numpy()
    assert np.linalg.norm(T @ aux - dv) <= 2e-7 * np.linalg.norm(dv)
    assert np.all(np.isfinite(dp.cpu().numpy()))


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


@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_qgt_onthefly_matvec_matches_dense(nk, dtype):
    """QGTOnTheFly (netket/optimizer/qgt/qgt_onthefly_logic.py:43-56): O_L v by the
    JVP kernel, O_L^T u by O^T v, S v = O_L^T O_L v + shift v, against the dense
    centred Jacobian (FP64: 1e-11 relative)."""
    N, n = 12, 600
    model, flat, M, x, t, p = _problem(nk, N, 2, n, seed=7)
    tt = t if dtype == "f64" else t.float()
    S = nk.ngd.QGTOnTheFly(tt, x, N, M, 1e-2)
    # the dense centred Jacobian of the same (FP32-rounded on the f32 path) t
    O_L = nk.kernels.jacobian_dense(tt.double(), x, N, M, S.obar, S.s, torch.float64)
    rng = np.random.default_rng(1)
    v = torch.as_tensor(rng.normal(size=O_L.shape[1]), device="cuda")
    u = torch.as_tensor(rng.normal(size=n), device="cuda")
    tol = 1e-11 if dtype == "f64" else 2e-6
    ref_ov = (O_L @ v).cpu().numpy()
    np.testing.assert_allclose(S.o_l(v).cpu().numpy(), ref_ov, rtol=tol, atol=tol * np.abs(ref_ov).max())
    ref_otu = (O_L.T @ u).cpu().numpy()
    np.testing.assert_allclose(S.o_l_t(u).cpu().numpy(), ref_otu, rtol=tol,
                               atol=tol * np.abs(ref_otu).max())
    ref_sv = (O_L.T @ (O_L @ v) + 1e-2 * v).cpu().numpy()
    np.testing.assert_allclose((S @ v).cpu().numpy(), ref_sv, rtol=tol, atol=tol * np.abs(ref_sv).max())


def test_sr_onthefly_cg_matches_dense_sr(nk):
    """SR with QGTOnTheFly + CG (NetKet's default for an RBM) converges to the
    dense-QGT Cholesky solution: to 1e-8 with a tight tolerance, and within the
    jax cg default (tol 1e-5) otherwise; warm start from the previous solution
    takes fewer iterations."""
    N, n = 16, 1008
    model, flat, M, x, t, p = _problem(nk, N, 1, n, seed=8)
    g = nk.graph.Chain(N)
    H = nk.operator.Ising(nk.hilbert.Spin(0.5, N), g, h=1.0, J=1.0)
    e = nk.kernels.local_energies_fused(H, flat, x, N, M)
    mean = e.mean().reshape(1)
    dense, _ = nk.ngd.sr_update(t, x, N, M, e, mean, 1e-2)
    d = dense.cpu().numpy()
    tight, info = nk.ngd.sr_update_onthefly(t, x, N, M, e, mean, 1e-2, tol=1e-12)
    np.testing.assert_allclose(tight.cpu().numpy(), d, rtol=1e-8, atol=1e-8 * np.abs(d).max())
    loose, info1 = nk.ngd.sr_update_onthefly(t, x, N, M, e, mean, 1e-2)
    assert np.linalg.norm(loose.cpu().numpy() - d) < 1e-3 * np.linalg.norm(d)
    warm, info2 = nk.ngd.sr_update_onthefly(t, x, N, M, e, mean, 1e-2, x0=loose)
    assert info2["cg_iterations"] <= 1 < info1["cg_iterations"]


def test_spring_minsr_and_sr_match_oracle(nk):
    """SPRING (netket/_src/ngd/srt.py:34-35, 63-66, 79-82; sr.py:43-47) against
    the oracle, which is pinned to the reference's own update functions."""
    N, n = 12, 256
    model, flat, M, x, t, p = _problem(nk, N, 2, n, seed=9)
    H = nk.operator.Heisenberg(nk.hilbert.Spin(0.5, N), nk.graph.Chain(N))
    e = nk.kernels.local_energies_fused(H, flat, x, N, M)
    mean = e.mean().reshape(1)
    P = M + N * M + N
    old = torch.as_tensor(np.random.default_rng(3).normal(scale=0.05, size=P), device="cuda")
    O = orbm.jacobian(p, x.cpu().numpy(), center=True)
    ec = e.cpu().numpy()
    for proj in (None, 0.5):
        dp, _ = nk.ngd.minsr_update(t, x, N, M, e, mean, 1e-3, proj_reg=proj, momentum=0.8,
                                    old_updates=old)
        dp = dp + 0.8 * old
        ref, _, _ = ongd.srt_update(O, ec, 1e-3, proj_reg=proj, momentum=0.8,
                                    old_updates=old.cpu().numpy())
        np.testing.assert_allclose(dp.cpu().numpy(), ref, rtol=1e-8, atol=1e-8 * np.abs(ref).max())
    dps, _ = nk.ngd.sr_update(t, x, N, M, e, mean, 1e-2, momentum=0.8, old_updates=old)
    refs, _, _ = ongd.sr_update(O, ec, 1e-2, momentum=0.8, old_updates=old.cpu().numpy())
    np.testing.assert_allclose(dps.cpu().numpy(), refs, rtol=1e-8, atol=1e-8 * np.abs(refs).max())
    # proj_reg only lifts the all-ones direction of the centred T, which the
    # centred dv does not touch: the update is unchanged
    a, _ = nk.ngd.minsr_update(t, x, N, M, e, mean, 1e-3)
    b, _ = nk.ngd.minsr_update(t, x, N, M, e, mean, 1e-3, proj_reg=2.0)
    np.testing.assert_allclose(b.cpu().numpy(), a.cpu().numpy(), rtol=1e-7,
                               atol=1e-9 * float(a.abs().max()))


def test_vmc_sr_spring_driver(nk):
    """VMC_SR(momentum=...): the first step equals the plain step bit for bit
    (old_updates starts at zero), later steps differ, old_updates is the last
    update; adding proj_reg changes only rounding (the centred minSR system does
    not see it); proj_reg is refused for SR as in the reference."""
    N = 10
    hi = nk.hilbert.Spin(0.5, N, total_sz=0)
    H = nk.operator.Heisenberg(hi, nk.graph.Chain(N))

    def make(**kw):
        vs = nk.vqs.MCState(nk.sampler.MetropolisExchange(hi, graph=nk.graph.Chain(N),
                                                          n_chains=64),
                            nk.models.RBM(alpha=2), n_samples=256, seed=5, precision="fp64")
        return vs, nk.driver.VMC_SR(H, nk.optimizer.Sgd(0.02), diag_shift=1e-3,
                                    variational_state=vs, use_ntk=True, **kw)

    vs_a, drv_a = make()
    vs_b, drv_b = make(momentum=lambda step: 0.8)
    drv_a.advance(1)
    drv_b.advance(1)
    assert torch.equal(vs_a.flat_parameters, vs_b.flat_parameters)
    drv_a.advance(1)
    drv_b.advance(1)
    assert not torch.equal(vs_a.flat_parameters, vs_b.flat_parameters)
    assert torch.equal(drv_b._old_updates, drv_b._dp)
    vs_p, drv_p = make(momentum=0.8, proj_reg=0.1)
    drv_p.advance(2)
    np.testing.assert_allclose(vs_p.flat_parameters.cpu().numpy(),
                               vs_b.flat_parameters.cpu().numpy(), rtol=1e-6, atol=1e-9)
    vs_s = nk.vqs.MCState(nk.sampler.MetropolisExchange(hi, graph=nk.graph.Chain(N),
                                                        n_chains=64),
                          nk.models.RBM(alpha=1), n_samples=512, seed=5, precision="fp64")
    drv_s = nk.driver.VMC_SR(H, nk.optimizer.Sgd(0.02), diag_shift=1e-3, variational_state=vs_s,
                             use_ntk=False, proj_reg=0.1)
    with pytest.raises(ValueError, match="proj_reg"):
        drv_s.advance(1)


def test_bounded_waits_run_out_and_recover(nk):
    """Device-side waits are bounded (vmck_set_wait_limit_ns).  With the limit
    shortened to 1 ns the tensor-core Gram (pipeline waits between its TMA, MMA
    and epilogue warps) and the refined solve (waits between the CTAs of the
    persistent triangular solves) wind down and report VMCK_DEV_TIMEOUT instead
    of hanging; with the default restored the next calls on the same context give
    the right results."""
    L = nk._native.lib()
    default = L.vmck_wait_limit_ns()
    assert default == 2_000_000_000
    N, alpha, n = 100, 4, 2048
    model, flat, M, x, t, p = _problem(nk, N, alpha, n)
    t32 = t.float().contiguous()
    obar = nk.kernels.column_means(t, x, N, M)
    st0 = torch.zeros(1, dtype=torch.int32, device="cuda")
    T64, T32 = nk.kernels.gram_structured(t32, x, N, M, obar, 1e-3, mode=2, want_f32=True,
                                          status=st0)
    assert st0.item() == 0
    T64, T32 = T64.clone(), T32.clone()
    ns = 8192
    rng = np.random.default_rng(5)
    U = rng.normal(size=(ns, 200))
    A = U @ U.T / 200 + 1e-3 * np.eye(ns)
    b = rng.normal(size=ns)
    At, bt = torch.as_tensor(A, device="cuda"), torch.as_tensor(b, device="cuda")
    try:
        L.vmck_set_wait_limit_ns(1)
        st = torch.zeros(1, dtype=torch.int32, device="cuda")
        nk.kernels.gram_structured(t32, x, N, M, obar, 1e-3, mode=2, want_f32=True, status=st)
        torch.cuda.synchronize()
        assert st.item() & nk._native.DEV_TIMEOUT
        st = torch.zeros(1, dtype=torch.int32, device="cuda")
        nk.kernels.cholesky_solve_refined(At, At.float().contiguous(), bt, st, max_iter=2)
        torch.cuda.synchronize()
        assert st.item() & nk._native.DEV_TIMEOUT
    finally:
        L.vmck_set_wait_limit_ns(default)
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    G64, G32 = nk.kernels.gram_structured(t32, x, N, M, obar, 1e-3, mode=2, want_f32=True,
                                          status=st)
    assert st.item() == 0
    low = torch.tril(torch.ones(n, n, dtype=torch.bool, device="cuda"))
    assert torch.equal(G64[low], T64[low]) and torch.equal(G32[low], T32[low])
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    xs, res = nk.kernels.cholesky_solve_refined(At, At.float().contiguous(), bt, st, max_iter=6)
    assert st.item() == 0 and res.item() < 1e-10
    ref = np.linalg.solve(A, b)
    np.testing.assert_allclose(xs.cpu().numpy(), ref, rtol=1e-9, atol=1e-9 * np.abs(ref).max())
