"""The allocation-free statistics entry point (vmck_stats_f64_noalloc), called
through the C ABI, against the workspace form (vmck_stats_f64) on the same
data.  It exists for callers that cannot allocate device memory mid-run (an
XLA FFI handler, a runtime whose pool owns the device); its scratch is a fixed
array inside the library, shared by every call, so this test makes two calls in
a row with different data and checks the second is not affected by the first.

This file is named to be collected last: a failure here leaves every other
test already run.  It also passes alone in a fresh process."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    from netket_gb300 import _native
    _native.require_cuda()
    return _native.lib()


def _with_workspace(L, data, plain):
    B, n = data.shape
    ws = torch.empty(L.vmck_stats_workspace_size(B, n), dtype=torch.float64, device="cuda")
    out = torch.empty(5, dtype=torch.float64, device="cuda")
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = L.vmck_stats_f64(s, ctypes.c_void_p(data.data_ptr()), B, n, plain,
                          ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(ws.data_ptr()), ws.numel())
    assert rc == 0, L.vmck_last_error()
    return out


def _no_alloc(L, data, plain):
    B, n = data.shape
    out = torch.empty(5, dtype=torch.float64, device="cuda")
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = L.vmck_stats_f64_noalloc(s, ctypes.c_void_p(data.data_ptr()), B, n, plain,
                                  ctypes.c_void_p(out.data_ptr()))
    assert rc == 0, L.vmck_last_error()
    return out


@pytest.mark.parametrize("shape,plain", [((4096, 4), 0), ((16, 63), 0), ((37, 129), 1)])
def test_noalloc_matches_workspace_form_twice(lib, shape, plain):
    g = torch.Generator(device="cuda").manual_seed(shape[0])
    for call in range(2):
        data = (torch.randn(shape, device="cuda", dtype=torch.float64, generator=g)
                * (1 + call) - 3.0 * call)
        ref = _with_workspace(lib, data, plain)
        got = _no_alloc(lib, data, plain)
        torch.cuda.synchronize()
        np.testing.assert_allclose(got.cpu().numpy(), ref.cpu().numpy(), rtol=1e-14, atol=0,
                                   equal_nan=True)


def test_noalloc_rejects_sizes_beyond_its_scratch(lib):
    data = torch.zeros((8192, 64), dtype=torch.float64, device="cuda")
    out = torch.zeros(5, dtype=torch.float64, device="cuda")
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = lib.vmck_stats_f64_noalloc(s, ctypes.c_void_p(data.data_ptr()), 8192, 64, 0,
                                    ctypes.c_void_p(out.data_ptr()))
    assert rc == 1 and b"scratch" in lib.vmck_last_error()
    torch.cuda.synchronize()
    assert torch.all(out == 0)
