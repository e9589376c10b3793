"""Host logic of the minSR fallback, without a GPU: after a failed factorisation
``minsr_fallback`` first solves the FP64 T by the shifted-factor PCG and takes
pinv_smooth (``cholesky_with_fallback``, netket/optimizer/solver/solvers.py:
305-340) only when that fails; ``try_pcg=False`` goes to pinv_smooth directly and
``pinv=False`` returns None (the driver's NaN for ``linear_solver="cholesky"``).
The device kernels are replaced by fakes that record the calls."""
import pytest
import torch

import netket_gb300 as nk
from netket_gb300 import ngd


class FakeKernels:
    def __init__(self, pcg_status):
        self.calls = []
        self.pcg_status = pcg_status

    def cholesky_solve_pcg(self, T, dv, st, tol, A32):
        self.calls.append(("pcg", tol, A32 is not None))
        st.fill_(self.pcg_status)
        return dv * 2.0, torch.tensor([1e-9], dtype=torch.float64), 0.5

    def pinv_smooth_solve(self, A, dv, rtol, rtol_smooth):
        assert torch.equal(A, A.T)  # the full symmetric matrix from the lower triangle
        self.calls.append(("pinv", rtol, rtol_smooth))
        return dv * 3.0

    def ot_v(self, t, x, N, M, aux):
        return aux.clone()

    def center_update(self, raw, obar, aux, s):
        return raw * s


def _info(n=4):
    T = torch.tril(torch.arange(1.0, n * n + 1, dtype=torch.float64).reshape(n, n))
    dv = torch.arange(1.0, n + 1, dtype=torch.float64)
    info = ngd.SolveInfo(solver_fallback=False)
    info["_fallback_args"] = (None, None, 2, 3, None, dv, T, 0.5, 1e-14, 1e-12)
    info["_pcg"] = (torch.zeros(n, n), 1e-8)
    info["status"] = nk._native.DEV_NOT_SPD | nk._native.DEV_NONFINITE  # a failed pivot
    return info, dv


@pytest.fixture
def fake(monkeypatch):
    def make(status):
        f = FakeKernels(status)
        monkeypatch.setattr(ngd, "K", f)
        monkeypatch.setattr(ngd, "_status", lambda: torch.zeros(1, dtype=torch.int32))
        return f
    return make


def test_pcg_solves_a_failed_factor(fake):
    f = fake(0)
    info, dv = _info()
    d = ngd.minsr_fallback(info)
    assert f.calls == [("pcg", 1e-8, True)]
    assert torch.equal(d, dv * 2.0 * 0.5) and torch.equal(info["aux"], dv * 2.0)
    assert not info["solver_fallback"]
    assert info["pcg"] == {"status": 0, "shift": 0.5, "residual": 1e-9}


@pytest.mark.parametrize("status", [nk._native.DEV_NOT_SPD, nk._native.DEV_NO_CONVERGE,
                                    nk._native.DEV_NONFINITE])
def test_pinv_smooth_when_pcg_fails(fake, status):
    f = fake(status)
    info, dv = _info()
    d = ngd.minsr_fallback(info)
    assert [c[0] for c in f.calls] == ["pcg", "pinv"]
    assert f.calls[1] == ("pinv", 1e-14, 1e-12)
    assert torch.equal(d, dv * 3.0 * 0.5) and info["solver_fallback"]
    assert info["pcg"]["status"] == status


def test_no_pinv_gives_none(fake):
    f = fake(nk._native.DEV_NOT_SPD)
    info, _ = _info()
    assert ngd.minsr_fallback(info, pinv=False) is None
    assert [c[0] for c in f.calls] == ["pcg"]
    assert not info["solver_fallback"]


def test_pinv_smooth_requested(fake):
    f = fake(0)
    info, dv = _info()
    d = ngd.minsr_fallback(info, try_pcg=False)
    assert [c[0] for c in f.calls] == ["pinv"]
    assert torch.equal(d, dv * 3.0 * 0.5) and "pcg" not in info


def test_dense_gram_has_no_pcg(fake):
    f = fake(0)
    info, _ = _info()
    del info["_pcg"]  # gram="dense": no structured T to precondition
    ngd.minsr_fallback(info)
    assert [c[0] for c in f.calls] == ["pinv"]
