"""Typed wrappers of the libvmck kernels on torch device tensors.

These are the building blocks the sampler, the variational state, the SR/minSR
solvers, the batched runner and the server share.  Every function launches on
torch's current CUDA stream and allocates its outputs with torch's caching
allocator; nothing here synchronises with the host.
"""
import ctypes
import math

import torch

from . import _native as nat


def _dev():
    return nat.device()


# ------------------------------------------------------------------ RBM forward
# FP32 contractions of at least this many sample x hidden-unit products run on
# the tensor cores (vmck_rbm_logpsi_tc / vmck_rbm_ot_v_tc); smaller ones on the
# CUDA cores, where the operand preparation would cost more than the product.
TC_MIN_WORK = 1 << 22


def _use_tc(dt, n, M, use_tc):
    if use_tc is None:
        return dt == torch.float32 and n * M >= TC_MIN_WORK
    if use_tc and dt != torch.float32:
        raise ValueError("the tensor-core RBM contractions take FP32 inputs")
    return bool(use_tc)


def rbm_forward(params_c, x, N, M, want_theta=False, want_tanh=False, use_tc=None):
    """logpsi (n,), optional theta and tanh(theta) (n, M), in params_c.dtype.
    ``use_tc``: None picks the tensor-core x W for large FP32 problems."""
    n = x.shape[0]
    dt = params_c.dtype
    lp = torch.empty(n, dtype=dt, device=x.device)
    th = torch.empty((n, M), dtype=dt, device=x.device) if want_theta else None
    tt = torch.empty((n, M), dtype=dt, device=x.device) if want_tanh else None
    if _use_tc(dt, n, M, use_tc):
        L = nat.lib()
        nb = L.vmck_rbm_logpsi_tc_workspace_size(N, M, n, int(th is not None))
        ws = torch.empty(nb, dtype=torch.uint8, device=x.device)
        nat.check(L.vmck_rbm_logpsi_tc(nat.stream(), nat.ptr(params_c), N, M, nat.ptr(x), n,
                                       nat.ptr(lp), nat.ptr(th), nat.ptr(tt), nat.ptr(ws), nb,
                                       None))
        return lp, th, tt
    nat.check(nat.lib().vmck_rbm_logpsi(nat.stream(), nat.dtype_code(dt), nat.ptr(params_c), N, M,
                                        nat.ptr(x), n, nat.ptr(lp), nat.ptr(th), nat.ptr(tt)))
    return lp, th, tt


# ------------------------------------------------------------------ local energies
def local_energies_fused(op, params_c, x, N, M):
    """E_loc (n,) FP64 via the fused log-ratio kernel (no connected states stored)."""
    from .operator import Ising, LocalOperator, PauliStrings
    n = x.shape[0]
    e = torch.empty(n, dtype=torch.float64, device=x.device)
    dt = nat.dtype_code(params_c.dtype)
    if isinstance(op, PauliStrings):
        st = op.device_struct()
        nat.check(nat.lib().vmck_rbm_eloc_pauli(nat.stream(), dt, nat.ptr(params_c), N, M,
                                                nat.ptr(x), n, ctypes.byref(st), nat.ptr(e), None))
        return e
    if isinstance(op, Ising):
        ed = op._edges_dev()
        nat.check(nat.lib().vmck_rbm_eloc_ising(nat.stream(), dt, nat.ptr(params_c), N, M,
                                                nat.ptr(x), n, nat.ptr(ed), len(op.edges), op.h,
                                                op.J, nat.ptr(e), None))
    elif isinstance(op, LocalOperator):
        st = op.device_struct()
        nat.check(nat.lib().vmck_rbm_eloc_local(nat.stream(), dt, nat.ptr(params_c), N, M,
                                                nat.ptr(x), n, ctypes.byref(st), nat.ptr(e), None))
    else:
        raise TypeError(f"no fused local-energy kernel for {type(op).__name__}")
    return e


def local_energies_dense(op, params_c, x, N, M, chunk=None):
    """E_loc the way NetKet computes it (``netket/vqs/mc/kernels.py:62-71``):
    get_conn_padded, logpsi of every connected row, then the reduction."""
    n = x.shape[0]
    dt = params_c.dtype
    e = torch.empty(n, dtype=torch.float64, device=x.device)
    K = op.max_conn_size if not hasattr(op, "h") or op.h != 0 else 1
    if chunk is None:
        chunk = max(1, min(n, (1 << 28) // max(1, K * (N + 8 + 8))))
    for s0 in range(0, n, chunk):
        xs = x[s0:s0 + chunk]
        xp, mels = op.get_conn_padded(xs)
        m = xs.shape[0]
        lp, _, _ = rbm_forward(params_c, xs, N, M)
        lpc, _, _ = rbm_forward(params_c, xp.reshape(-1, N), N, M)
        nat.check(nat.lib().vmck_eloc_from_logpsi(nat.stream(), nat.dtype_code(dt), nat.ptr(lp),
                                                  nat.ptr(lpc), nat.ptr(mels), m,
                                                  mels.shape[1], nat.ptr(e[s0:s0 + m])))
    return e


# ------------------------------------------------------------------ statistics
def stats_device(data2d, plain_rhat=False):
    """[mean, error_of_mean, variance, tau_corr, R_hat] (5,) FP64 on the device."""
    B, L = data2d.shape
    d = data2d.to(torch.float64).contiguous()
    ws = torch.empty(max(1, nat.lib().vmck_stats_workspace_size(B, L)), dtype=torch.float64,
                     device=d.device)
    out = torch.empty(5, dtype=torch.float64, device=d.device)
    nat.check(nat.lib().vmck_stats_f64(nat.stream(), nat.ptr(d), B, L, int(plain_rhat),
                                       nat.ptr(out), nat.ptr(ws), ws.numel()))
    return out


def online_stats_update(data2d, state, max_lag, buf_len, decay, mean_f32):
    """Merge ``data2d`` (n_chains, n_batch) FP64 into the accumulator tensors
    ``state`` (dict count/mean/M2/cross/m1/m2/pair/buf, FP64, on the device) in
    place; see ``vmck_online_stats_update``."""
    C, nb = data2d.shape
    d = data2d.to(torch.float64).contiguous()
    st = nat.OnlineStatsStruct(*[nat.ptr(state[k]) if state[k].numel() else None
                                 for k in ("count", "mean", "M2", "cross", "m1", "m2", "pair",
                                           "buf")])
    nat.check(nat.lib().vmck_online_stats_update(nat.stream(), nat.ptr(d), C, nb, int(max_lag),
                                                 int(buf_len), float(decay), int(mean_f32),
                                                 ctypes.byref(st)))


# ------------------------------------------------------------------ Jacobian products
def ot_v(tanh_t, x, N, M, v, use_tc=None):
    """O^T v (P,) FP64 for the RBM Jacobian, never materialising O.  ``use_tc``:
    None picks the tensor-core GEMM for large FP32 problems."""
    n = x.shape[0]
    P = M + N * M + N
    out = torch.empty(P, dtype=torch.float64, device=x.device)
    if _use_tc(tanh_t.dtype, n, M, use_tc):
        L = nat.lib()
        nb = L.vmck_rbm_ot_v_tc_workspace_size(N, M, n)
        ws = torch.empty(nb, dtype=torch.uint8, device=x.device)
        nat.check(L.vmck_rbm_ot_v_tc(nat.stream(), nat.ptr(tanh_t), nat.ptr(x), N, M, n,
                                     nat.ptr(v.contiguous()), nat.ptr(out), nat.ptr(ws), nb, None))
        return out
    ws = torch.empty(nat.lib().vmck_ot_v_workspace_size(N, M, n), dtype=torch.float64,
                     device=x.device)
    nat.check(nat.lib().vmck_rbm_ot_v(nat.stream(), nat.dtype_code(tanh_t.dtype), nat.ptr(tanh_t),
                                      nat.ptr(x), N, M, n, nat.ptr(v.contiguous()), nat.ptr(out),
                                      nat.ptr(ws), ws.numel()))
    return out


def o_v(tanh_t, x, N, M, v):
    """O v (n,) FP64 for the RBM Jacobian (the JVP of QGTOnTheFly), O never stored."""
    n = x.shape[0]
    out = torch.empty(n, dtype=torch.float64, device=x.device)
    nat.check(nat.lib().vmck_rbm_o_v(nat.stream(), nat.dtype_code(tanh_t.dtype), nat.ptr(tanh_t),
                                     nat.ptr(x), N, M, n, nat.ptr(v.contiguous()), nat.ptr(out)))
    return out


def column_means(tanh_t, x, N, M):
    n = x.shape[0]
    v = torch.full((n,), 1.0 / n, dtype=torch.float64, device=x.device)
    return ot_v(tanh_t, x, N, M, v)


def jacobian_dense(tanh_t, x, N, M, col_mean, scale, out_dtype):
    n = x.shape[0]
    P = M + N * M + N
    O = torch.empty((n, P), dtype=out_dtype, device=x.device)
    nat.check(nat.lib().vmck_rbm_jacobian(nat.stream(), nat.dtype_code(tanh_t.dtype),
                                          nat.ptr(tanh_t), nat.ptr(x), N, M, n, nat.ptr(col_mean),
                                          float(scale), nat.dtype_code(out_dtype), nat.ptr(O)))
    return O


def gram_structured(tanh_t, x, N, M, obar, diag_shift, mode, want_f32=False, status=None):
    """Lower triangle of T = O_L O_L^T + diag_shift I (n, n) FP64 (+ FP32 copy).
    mode 0: FP64 CUDA cores; 1: FP32 CUDA cores; 2: tcgen05 BF16 hi/lo split;
    3: tcgen05 single BF16; 4: tcgen05 FP16 hi/lo split (four products) with per-slab drained
    accumulation (the blocked-Cholesky GEMM) and a double-float assembly pass."""
    n = x.shape[0]
    T64 = torch.empty((n, n), dtype=torch.float64, device=x.device)
    T32 = torch.empty((n, n), dtype=torch.float32, device=x.device) if want_f32 else None
    ws = torch.empty(nat.lib().vmck_gram_workspace_size(N, M, n), dtype=torch.float64,
                     device=x.device)
    nat.check(nat.lib().vmck_rbm_gram(nat.ctx(), nat.stream(), int(mode),
                                      nat.dtype_code(tanh_t.dtype), nat.ptr(tanh_t), nat.ptr(x), N,
                                      M, n, nat.ptr(obar), float(diag_shift), nat.ptr(T64),
                                      nat.ptr(T32), nat.ptr(ws), ws.numel(), nat.ptr(status)))
    return T64, T32


def gram_dense(O_L, diag_shift, transpose=False):
    rows, cols = O_L.shape
    m = cols if transpose else rows
    out = torch.empty((m, m), dtype=O_L.dtype, device=O_L.device)
    nat.check(nat.lib().vmck_gram_dense(nat.ctx(), nat.stream(), nat.dtype_code(O_L.dtype),
                                        nat.ptr(O_L), rows, cols, int(transpose),
                                        float(diag_shift), nat.ptr(out)))
    return out


# ------------------------------------------------------------------ solvers
def cholesky_solve(A, b, status):
    x = torch.empty_like(b)
    nat.check(nat.lib().vmck_cholesky_solve(nat.ctx(), nat.stream(), nat.dtype_code(A.dtype),
                                            nat.ptr(A), nat.ptr(b), nat.ptr(x), A.shape[0],
                                            nat.ptr(status)))
    return x


def cholesky_solve_refined(A64, A32, b, status, max_iter=3, tol=1e-10, factor_mode=4):
    """FP32-accurate Cholesky of A32 (overwritten by its factor) refined to an
    FP64 residual against A64.  factor_mode 4 (default): this library's blocked
    factorisation on the tcgen05 tensor cores (FP16 hi + lo operand split, FP32
    accumulation) with its own leaf, panel and trailing-update kernels.  For
    comparison: 0 cuSOLVER SPOTRF; 1 SPOTRF with BF16x9 emulation; 2 recursive
    GEMM factorisation on BF16x9-emulated cuBLAS; 3 blocked factorisation with
    the library's 128 x 128 leaf and emulated cuBLAS GEMMs."""
    x = torch.empty_like(b)
    res = torch.empty(1, dtype=torch.float64, device=b.device)
    nat.check(nat.lib().vmck_cholesky_solve_refined(nat.ctx(), nat.stream(), nat.ptr(A64),
                                                    nat.ptr(A32), nat.ptr(b), nat.ptr(x),
                                                    A64.shape[0], int(max_iter), float(tol),
                                                    int(factor_mode), nat.ptr(status),
                                                    nat.ptr(res)))
    return x, res


def cholesky_solve_pcg(A64, b, status, max_iter=2000, tol=1e-10, shift_rel=1e-7, A32=None):
    """Solution of A64 x = b (A64 SPD, lower triangle set) when its FP32 factor
    fails: the tensor-core factor of A + mu I (mu = shift_rel trace(A), x16 per
    failed attempt) preconditions flexible CG with FP64 products of A64.
    Returns (x, relative residual (device), mu).  A32 (optional, n x n FP32) is
    used as the factor's storage.  Synchronises the stream."""
    x = torch.empty_like(b)
    res = torch.zeros(1, dtype=torch.float64, device=b.device)
    mu = ctypes.c_double(0.0)
    nat.check(nat.lib().vmck_cholesky_solve_pcg(
        nat.ctx(), nat.stream(), nat.ptr(A64), nat.ptr(A32) if A32 is not None else None,
        nat.ptr(b), nat.ptr(x), A64.shape[0], int(max_iter), float(tol), float(shift_rel),
        nat.ptr(status), nat.ptr(res), ctypes.byref(mu)))
    return x, res, mu.value


def pinv_smooth_solve(A, b, rtol=1e-14, rtol_smooth=1e-14):
    x = torch.empty_like(b)
    nat.check(nat.lib().vmck_pinv_smooth_solve(nat.ctx(), nat.stream(), nat.ptr(A), nat.ptr(b),
                                               nat.ptr(x), A.shape[0], float(rtol),
                                               float(rtol_smooth)))
    return x


def center_scale(e, mean_dev, factor):
    out = torch.empty_like(e)
    nat.check(nat.lib().vmck_center_scale(nat.stream(), nat.ptr(e), nat.ptr(mean_dev), e.numel(),
                                          float(factor), nat.ptr(out)))
    return out


def center_update(raw, obar, aux, scale):
    out = torch.empty_like(raw)
    nat.check(nat.lib().vmck_center_update(nat.stream(), nat.ptr(raw), nat.ptr(obar),
                                           nat.ptr(aux), aux.numel(), raw.numel(), float(scale),
                                           nat.ptr(out)))
    return out


def sgd_(p64, update, lr, p32=None):
    nat.check(nat.lib().vmck_sgd(nat.stream(), nat.ptr(p64), nat.ptr(update), p64.numel(),
                                 float(lr), nat.ptr(p32)))


def cast_f32(src, out=None):
    out = torch.empty(src.shape, dtype=torch.float32, device=src.device) if out is None else out
    nat.check(nat.lib().vmck_cast_f64_f32(nat.stream(), nat.ptr(src), nat.ptr(out), src.numel()))
    return out


def inv_sqrt(n):
    return 1.0 / math.sqrt(n)
