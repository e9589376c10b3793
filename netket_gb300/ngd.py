"""SR / minSR natural-gradient updates on the GPU.

``minsr_update`` is ``netket/_src/ngd/srt.py:22-96`` (with ``_prepare_input``,
``netket/_src/ngd/sr_srt_common.py:45-101``): ``T = O_L O_L^T + lambda I``,
``aux = T^-1 dv``, ``delta = O_L^T aux`` with ``O_L = (O - mean O)/sqrt(n)`` and
``dv = 2 (E - mean E)/sqrt(n)``.  ``sr_update`` is ``netket/_src/ngd/sr.py:23-80``.

Two ways to form T:
  * ``gram="structured"`` (default): the RBM identity
    ``O(s).O(s') = (t_s.t_s')(1 + x_s.x_s') + x_s.x_s'`` (t = tanh theta) turns
    the (n x n x P) contraction into (n x n x M), and O is never stored.  For an
    FP32 t the contraction is shifted by the column mean and the shift is added
    back in double-float (no cancellation).  ``gram_mode=4`` (default) contracts
    on the tensor cores (tcgen05) with t - s0 on a 2^-19 grid split into
    fixed-point FP16 hi + lo (all four products, so T is the Gram matrix of
    that Jacobian; every 64-wide slab of hi * hi sums exactly and the slabs add
    in FP32 registers), then a double-float assembly pass; ``2`` rounds t to hi +
    lo BF16 pairs and accumulates in tensor memory over the whole K (its T lost
    positive definiteness at M = 2048: the accumulation error grows with the MMA
    chain), ``3`` one BF16, ``1`` FP32 on the CUDA cores.  At the 10 x 10 alpha-4
    workload (n = 4,096, diag_shift 1e-4) the minSR update of mode 4 is within
    1.1e-5 (relative) of the all-FP64 one, mode 2 within 2.9e-5; at n = 16,384
    mode 4 takes 2.0 ms for T, mode 2 2.5 ms;
  * ``gram="dense"``: the reference algorithm, a materialised (n, P) Jacobian
    and a cuBLAS SYRK.
Solvers (``solve=``):
  * ``"cholesky"``: Cholesky in the Jacobian's precision (FP64: this library's
    tensor-core FP32 factor refined with the FP64 residual to FP64 rounding;
    FP32: cuSOLVER, the plain path);
  * ``"refined"``: FP32 Cholesky (this library's tensor-core factorisation)
    refined against the FP64 matrix (iterative refinement) until the relative
    FP64 residual is below ``refine_tol`` (default 1e-8, at most ``refine_iters``
    correction solves; the loop stops on the device once it is reached).  The
    residual bound matters little beyond that: with T = O_L O_L^T + lambda I a
    residual r moves delta = O_L^T aux by at most |r| / (2 sqrt(lambda)), and the
    mixed path's Gram rounding already puts delta ~3e-5 (relative) from the
    all-FP64 update;
with NetKet's ``cholesky_with_fallback`` behaviour: a failed factorisation or a
non-finite result switches to ``pinv_smooth`` (``netket/optimizer/solver/
solvers.py:305-340``).
"""
import math

import torch

from . import _native as nat
from . import kernels as K


class SolveInfo(dict):
    pass


def _status():
    return torch.zeros(1, dtype=torch.int32, device=nat.device())


# FP32 Jacobians with M up to this use gram_mode 2 by default, larger ones mode 4
# (0: mode 4 everywhere -- faster and closer to FP64 at every size measured)
TC_GRAM_MAX_M = 0


def _o_l_v(t, x, N, M, obar, s, v):
    """O_L v = (O v - (obar . v) 1) / sqrt(n) by the JVP kernel."""
    return (K.o_v(t, x, N, M, v) - torch.dot(obar, v)) * s


def minsr_update(t, x, N, M, e, mean_dev, diag_shift, *, gram="structured", gram_mode=None,
                 solve="cholesky", refine_iters=4, refine_tol=1e-8, rtol=1e-14,
                 rtol_smooth=1e-14, jac_dtype=None, check=True, phase_timer=None,
                 proj_reg=None, momentum=None, old_updates=None):
    """Returns (delta (P,) FP64, info).  ``t`` = tanh(theta) (n, M) in the compute
    dtype, ``e`` = local energies (n,) FP64, ``mean_dev`` = their mean (device).

    With ``check=False`` the device status is not read here: ``info["status_dev"]``
    holds it and ``minsr_fallback(info)`` recomputes delta (shifted-factor PCG,
    then pinv_smooth) if the
    caller finds a failed factorisation (one host read per step).

    SPRING (``netket/_src/ngd/srt.py:34-35, 63-66``): ``proj_reg`` adds
    ``proj_reg / n`` to every entry of T; ``momentum`` with ``old_updates``
    subtracts ``momentum O_L old`` from dv.  The caller adds ``momentum old`` to
    the returned delta (after any fallback) and keeps the sum as the next
    ``old_updates``."""
    ph = phase_timer
    n = x.shape[0]
    s = 1.0 / math.sqrt(n)
    mode = None
    if gram == "structured":
        if gram_mode is not None:
            mode = gram_mode
        elif t.dtype == torch.float64:
            mode = 0
        else:
            mode = 2 if M <= TC_GRAM_MAX_M else 4
    obar = K.column_means(t, x, N, M)
    dv = K.center_scale(e, mean_dev, 2.0 * s)
    if momentum is not None and old_updates is not None:
        # SPRING (netket/_src/ngd/srt.py:34-35): dv -= momentum O_L old
        dv = dv - momentum * _o_l_v(t, x, N, M, obar, s, old_updates)
    status = _status()
    info = SolveInfo(solver_fallback=False)
    if gram == "structured":
        T64, T32 = K.gram_structured(t, x, N, M, obar, diag_shift, mode,
                                     want_f32=(solve == "refined" or mode >= 2), status=status)
        if proj_reg is not None:
            # T + proj_reg / n 1 1^T (netket/_src/ngd/srt.py:63-66)
            T64.add_(proj_reg / n)
            if T32 is not None:
                T32.add_(proj_reg / n)
        if ph:
            ph.mark("gram")
        if solve == "refined":
            aux, res = K.cholesky_solve_refined(T64, T32, dv, status, refine_iters, refine_tol)
            info["residual_dev"] = res
        else:
            aux = K.cholesky_solve(T64, dv, status)
        Tfb = T64
    elif gram == "dense":
        jd = jac_dtype or t.dtype
        O_L = K.jacobian_dense(t, x, N, M, obar, s, jd)
        T = K.gram_dense(O_L, diag_shift)
        if proj_reg is not None:
            T.add_(proj_reg / n)
        del O_L
        if ph:
            ph.mark("gram")
        if T.dtype == torch.float64:
            aux = K.cholesky_solve(T, dv, status)
        else:
            aux = K.cholesky_solve(T, dv.to(torch.float32), status).to(torch.float64)
        Tfb = T
    else:
        raise ValueError("gram must be 'structured' or 'dense'")
    info["status_dev"] = status
    if ph:
        ph.mark("solve")
    info["_fallback_args"] = (t, x, N, M, obar, dv, Tfb, s, rtol, rtol_smooth)
    if gram == "structured":
        # the FP64 system of a failed FP32 factor: shifted-factor PCG first
        info["_pcg"] = (T32, refine_tol if solve == "refined" else 1e-10)
    if check:
        st = int(status.item())
        info["status"] = st
        if st & (nat.DEV_NOT_SPD | nat.DEV_NONFINITE) or (
                solve == "cholesky" and st & nat.DEV_NO_CONVERGE):
            return minsr_fallback(info), info
    raw = K.ot_v(t, x, N, M, aux)
    delta = K.center_update(raw, obar, aux, s)
    if ph:
        ph.mark("update")
    return delta, info


def minsr_fallback(info, try_pcg=True, pinv=True):
    """delta after a failed solve (``try_pcg=False``: pinv_smooth directly;
    ``pinv=False``: None where pinv_smooth would be the answer).  The FP64
    Cholesky of the reference solves T up to cond(T) ~ 1e15; the FP32 factor
    here stops near 1e7.  So a failed
    factor of a finite, structured T is first retried as shifted-factor PCG
    against the FP64 T (``kernels.cholesky_solve_pcg``: the FP64 solution);
    only if that fails too -- T not positive definite, or not finite -- does it
    switch to pinv_smooth as ``cholesky_with_fallback`` does
    (``netket/optimizer/solver/solvers.py:305-340``)."""
    t, x, N, M, obar, dv, T, s, rtol, rtol_smooth = info["_fallback_args"]
    # (a failed pivot also reads as non-finite: the PCG itself reports a T that is)
    if try_pcg and "_pcg" in info and T.dtype == torch.float64:
        T32, tol = info["_pcg"]
        pst = _status()
        aux, res, mu = K.cholesky_solve_pcg(T, dv, pst, tol=tol, A32=T32)
        pst = int(pst.item())
        info["pcg"] = {"status": pst, "shift": mu, "residual": float(res.item())}
        if pst == 0:
            info["aux"] = aux
            raw = K.ot_v(t, x, N, M, aux)
            return K.center_update(raw, obar, aux, s)
    if not pinv:
        return None
    A = T.to(torch.float64)
    A = torch.tril(A) + torch.tril(A, -1).T
    aux = K.pinv_smooth_solve(A.contiguous(), dv, rtol, rtol_smooth)
    info["solver_fallback"] = True
    raw = K.ot_v(t, x, N, M, aux)
    return K.center_update(raw, obar, aux, s)


def sr_update(t, x, N, M, e, mean_dev, diag_shift, *, jac_dtype=None, rtol=1e-14,
              rtol_smooth=1e-14, momentum=None, old_updates=None):
    """SR with the dense QGT: (O_L^T O_L + lambda I) delta = O_L^T dv; with
    ``momentum``, ``F += diag_shift momentum old`` (netket/_src/ngd/sr.py:43-47)."""
    n = x.shape[0]
    s = 1.0 / math.sqrt(n)
    obar = K.column_means(t, x, N, M)
    dv = K.center_scale(e, mean_dev, 2.0 * s)
    raw = K.ot_v(t, x, N, M, dv)
    F = K.center_update(raw, obar, dv, s)
    if momentum is not None and old_updates is not None:
        F = F + (diag_shift * momentum) * old_updates
    jd = jac_dtype or torch.float64
    O_L = K.jacobian_dense(t, x, N, M, obar, s, jd)
    S = K.gram_dense(O_L, diag_shift, transpose=True)
    return solve_with_fallback(S.to(torch.float64), F, rtol, rtol_smooth)


class QGTOnTheFly:
    """``S v = O_L^T (O_L v) + diag_shift v`` without forming O or S
    (``netket/optimizer/qgt/qgt_onthefly_logic.py:43-56``): ``O v`` by the
    ``vmck_rbm_o_v`` JVP kernel, ``O^T w`` by ``vmck_rbm_ot_v``, both centred
    with the column means (``O_L = (O - 1 obar^T) / sqrt(n)``)."""

    def __init__(self, t, x, N, M, diag_shift):
        self.t, self.x, self.N, self.M = t, x, N, M
        self.n = x.shape[0]
        self.s = 1.0 / math.sqrt(self.n)
        self.diag_shift = diag_shift
        self.obar = K.column_means(t, x, N, M)

    def o_l(self, v):
        """O_L v (n,)."""
        w = K.o_v(self.t, self.x, self.N, self.M, v)
        return (w - torch.dot(self.obar, v)) * self.s

    def o_l_t(self, u):
        """O_L^T u (P,)."""
        raw = K.ot_v(self.t, self.x, self.N, self.M, u)
        return K.center_update(raw, self.obar, u, self.s)

    def __matmul__(self, v):
        return self.o_l_t(self.o_l(v)) + self.diag_shift * v


def cg(A, b, x0=None, tol=1e-5, atol=0.0, maxiter=None):
    """Conjugate gradients with ``jax.scipy.sparse.linalg.cg``'s stopping rule
    (``|r| <= max(tol |b|, atol)``, ``maxiter`` = 10 * size by default), the
    solver NetKet's ``SR`` uses by default.  Returns (x, iterations)."""
    x = torch.zeros_like(b) if x0 is None else x0.clone()
    maxiter = 10 * b.numel() if maxiter is None else maxiter
    bound2 = max(tol * tol * float(torch.dot(b, b)), atol * atol)
    r = b - A @ x
    p = r.clone()
    gamma = float(torch.dot(r, r))
    k = 0
    while gamma > bound2 and k < maxiter:
        Ap = A @ p
        alpha = gamma / float(torch.dot(p, Ap))
        x += alpha * p
        r -= alpha * Ap
        gamma_new = float(torch.dot(r, r))
        p = r + (gamma_new / gamma) * p
        gamma = gamma_new
        k += 1
    return x, k


def sr_update_onthefly(t, x, N, M, e, mean_dev, diag_shift, *, x0=None, tol=1e-5, atol=0.0,
                       maxiter=None):
    """SR with ``QGTOnTheFly`` and CG (NetKet's defaults for an RBM:
    ``netket/optimizer/qgt/default.py:58-97``, ``netket/optimizer/sr.py:62-216``).
    Returns (delta (P,), info with the CG iteration count)."""
    n = x.shape[0]
    S = QGTOnTheFly(t, x, N, M, diag_shift)
    dv = K.center_scale(e, mean_dev, 2.0 * S.s)
    F = S.o_l_t(dv)
    delta, iters = cg(S, F, x0=x0, tol=tol, atol=atol, maxiter=maxiter)
    info = SolveInfo(solver_fallback=False)
    info["cg_iterations"] = iters
    return delta, info


def solve_with_fallback(A, b, rtol=1e-14, rtol_smooth=1e-14):
    """``cholesky_with_fallback`` for an SPD matrix whose lower triangle is set."""
    status = _status()
    x = K.cholesky_solve(A, b, status)
    info = SolveInfo(solver_fallback=False)
    st = int(status.item())
    # the FP64 solve refines an FP32 factor; a refinement that does not converge
    # (cond(A) beyond the FP32 factor's reach) counts as a failed factorisation
    bad = nat.DEV_NOT_SPD | nat.DEV_NONFINITE
    if A.dtype == torch.float64:
        bad |= nat.DEV_NO_CONVERGE
    if st & bad:
        full = torch.tril(A) + torch.tril(A, -1).T
        x = K.pinv_smooth_solve(full.contiguous(), b, rtol, rtol_smooth)
        info["solver_fallback"] = True
    info["status"] = st
    return x, info
