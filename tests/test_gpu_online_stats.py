"""Streaming statistics on the GPU (vmck_online_stats_update) against the
reference-generated golden vectors and the FP64 oracle.

Tolerances: the accumulator arrays are FP64 sums whose summation order differs
from the reference's (per-lane sequential vs XLA reductions): 1e-13 relative to
the largest entry of each array.  Read-outs 1e-11 relative.  The ACF, formed
from raw moment sums as in the reference, 1e-13 x max(1, mean^2 / variance)
absolute (the cancellation in sum x_t x_{t-k} - sum x_{t-k} sum x_t / n)."""
import math

import numpy as np
import pytest
import torch

from oracle import online_stats as oos
from oracle import stats as ost

pytestmark = pytest.mark.gpu

KEYS = ("count", "mean", "M2", "cross", "m1", "m2", "pair", "buf")


@pytest.fixture(scope="module")
def nk():
    import netket_gb300
    netket_gb300._native.require_cuda()
    return netket_gb300


def run_gpu(nk, data, lens, max_lag, decay):
    est = None
    for ch in np.split(data, np.cumsum(lens)[:-1], axis=1):
        est = nk.stats.online_statistics(torch.as_tensor(ch, device="cuda"), est, decay=decay,
                                         max_lag=max_lag)
    return est


def run_oracle(data, lens, max_lag, decay):
    s = oos.new_state(data.shape[0], max_lag)
    for ch in np.split(data, np.cumsum(lens)[:-1], axis=1):
        s = oos.update(s, ch, decay)
    return s


def assert_state(est, ref, what=""):
    for k in KEYS:
        got = est._s[k].cpu().numpy()
        r = ref[k]
        scale = max(1.0, float(np.abs(r).max())) if r.size else 1.0
        np.testing.assert_allclose(got, r, rtol=0, atol=1e-13 * scale, err_msg=f"{what} {k}")
    assert est._buf_len == ref["buf_len"]


def acf_tol(data):
    return 1e-13 * max(1.0, float(np.mean(data)) ** 2 / float(np.var(data)))


@pytest.mark.parametrize("name", ["iid_oneshot", "iid_chunks", "ar1_small_batches",
                                  "ar1_ragged", "big_then_small", "decay", "no_acf",
                                  "one_chain", "shifted_mean"])
def test_online_stats_golden(nk, golden, name):
    """The device accumulator after the same chunk sequence as the reference's
    own _update_arrays run, and its read-outs."""
    g = golden("online_stats")
    data, lens, cfg = g[name + "__data"], g[name + "__lens"], g[name + "__cfg"]
    decay = None if cfg[1] < 0 else float(cfg[1])
    est = run_gpu(nk, data, lens, int(cfg[0]), decay)
    ref = {k: g[f"{name}__{k}"] for k in KEYS}
    ref["buf_len"] = int(g[name + "__buf_len"])
    assert_state(est, ref, name)
    st = est.get_stats()
    got = np.array([est.mean, est.variance, est.tau_corr, est.tau_corr_batch, est.tau_corr_acf,
                    est.R_hat, st.error_of_mean])
    np.testing.assert_allclose(got, g[name + "__derived"], rtol=1e-11, atol=1e-13,
                               equal_nan=True)
    ga = g[name + "__acf"]
    if ga.size == 0:
        assert est.acf is None
    else:
        np.testing.assert_allclose(est.acf.cpu().numpy(), ga, rtol=0, atol=acf_tol(data))


@pytest.mark.parametrize("C,lens,max_lag,decay", [
    (4096, [4] * 6, 64, None),            # expect_to_precision shape: 4 samples per chain per round
    (1000, [1, 1, 2, 3, 5, 8, 13], 33, None),
    (257, [31, 32, 33], 32, None),
    (64, [100, 7], 200, None),            # max_lag spans several 32-lag rounds per lane
    (3, [70, 1, 64], 64, 0.5),
    (16384, [2, 2], 0, None),             # ACF off
    (5, [40], 1, None),
])
def test_online_stats_vs_oracle(nk, C, lens, max_lag, decay):
    rng = np.random.default_rng(C + max_lag)
    data = rng.standard_normal((C, sum(lens))) * 2.0 + 0.3
    est = run_gpu(nk, data, lens, max_lag, decay)
    ref = run_oracle(data, lens, max_lag, decay)
    assert_state(est, ref, f"C={C} L={max_lag}")
    np.testing.assert_allclose([est.mean, est.variance, est.R_hat], oos.derived(ref)[[0, 1, 5]],
                               rtol=1e-11, equal_nan=True)
    assert est.n_samples == data.size


def test_online_stats_reference_properties(nk):
    """The reference test suite's properties (test/stats/test_online_stats.py)."""
    rng = np.random.default_rng(42)
    data = rng.standard_normal((64, 500))
    # chunked == one shot; mean / variance / error of the mean == batch statistics
    full = nk.stats.online_statistics(data)
    chunked = None
    for ch in np.split(data, 5, axis=1):
        chunked = nk.stats.online_statistics(ch, chunked)
    for a, b in [(full.mean, chunked.mean), (full.variance, chunked.variance),
                 (full.get_stats().error_of_mean, chunked.get_stats().error_of_mean)]:
        np.testing.assert_allclose(a, b, rtol=1e-10)
    bs = ost.statistics(data)
    np.testing.assert_allclose(full.mean, bs.mean, rtol=1e-10)
    np.testing.assert_allclose(full.variance, bs.variance, rtol=1e-10)
    np.testing.assert_allclose(full.get_stats().error_of_mean, bs.error_of_mean, rtol=1e-10)
    # ACF chunked vs one shot
    d4 = rng.standard_normal((4, 300))
    a = nk.stats.online_statistics(d4, max_lag=32)
    b = None
    for ch in np.split(d4, 10, axis=1):
        b = nk.stats.online_statistics(ch, b, max_lag=32)
    np.testing.assert_allclose(a.acf.cpu().numpy(), b.acf.cpu().numpy(), atol=1e-12)
    assert a.acf.shape == (33,) and abs(float(a.acf[0]) - 1.0) < 1e-12
    # R-hat: diverging chains vs iid chains
    div = np.vstack([rng.standard_normal((4, 100)), rng.standard_normal((4, 100)) + 10.0])
    assert nk.stats.online_statistics(div).R_hat > 1.01
    assert nk.stats.online_statistics(rng.standard_normal((16, 500))).R_hat < 1.1
    # AR(1), phi = 0.8: tau well above 1
    ar = np.zeros((8, 512))
    ar[:, 0] = rng.standard_normal(8)
    for t in range(1, 512):
        ar[:, t] = 0.8 * ar[:, t - 1] + math.sqrt(1 - 0.64) * rng.standard_normal(8)
    est = nk.stats.online_statistics(ar, max_lag=64)
    assert est.tau_corr_acf > 2.0 and math.isfinite(est.tau_corr_acf)
    assert est.tau_corr == est.tau_corr_acf
    # decay forgets old data
    e = None
    for _ in range(20):
        e = nk.stats.online_statistics(rng.standard_normal((4, 50)), e, decay=0.01)
    for _ in range(20):
        e = nk.stats.online_statistics(rng.standard_normal((4, 50)) + 10.0, e, decay=0.01)
    assert abs(e.mean - 10.0) < 0.5
    # single 1D chain: R-hat undefined, tau from the ACF
    one = nk.stats.online_statistics(rng.standard_normal(200))
    assert math.isnan(one.R_hat) and math.isfinite(one.tau_corr)
    assert math.isnan(nk.stats.online_statistics(rng.standard_normal(200), max_lag=0).tau_corr)
    # large batch fills the buffer with the newest samples
    big = rng.standard_normal((4, 12))
    est = nk.stats.online_statistics(big, max_lag=8)
    np.testing.assert_array_equal(est._chain_buf.cpu().numpy(), big[:, -8:])
    # immutability, chain-count check, float32 means kept in float32
    e1 = nk.stats.online_statistics(rng.standard_normal((4, 50)))
    c1 = float(e1._chain_count.sum())
    e2 = e1.update(rng.standard_normal((4, 50)))
    assert float(e1._chain_count.sum()) == c1 < float(e2._chain_count.sum())
    with pytest.raises(ValueError, match="Number of chains"):
        e1.update(rng.standard_normal((8, 10)))
    f32 = nk.stats.OnlineStats.from_data(rng.standard_normal((4, 100)).astype(np.float32))
    assert f32._chain_mean.dtype == torch.float32
    with pytest.raises(TypeError):
        nk.stats.online_statistics(rng.standard_normal((4, 10)) + 1j)


def test_online_stats_window_ops_then_update(nk):
    """expand_max_lag then further updates: the new lags collect pairs and the
    state equals the oracle's for the same operations."""
    rng = np.random.default_rng(77)
    b1 = rng.standard_normal((4, 100))
    est = nk.stats.expand_max_lag(nk.stats.online_statistics(b1, max_lag=16), 64)
    s = oos.update(oos.new_state(4, 16), b1)
    # the oracle's expansion: zero columns for new lags, left-padded buffer
    s = dict(s, max_lag=64, buf=np.pad(s["buf"], ((0, 0), (48, 0))),
             **{k: np.pad(s[k], ((0, 0), (0, 48))) for k in ("cross", "m1", "m2", "pair")})
    for _ in range(5):
        b = rng.standard_normal((4, 50))
        est = est.update(b)
        s = oos.update(s, b)
    assert_state(est, s, "expanded")
    assert float(est._pair_count[:, 20:].sum()) > 0
    th = nk.stats.thin_acf_by_2(est)
    th = th.update(rng.standard_normal((4, 3)))
    assert th.max_lag == 32 and th.acf.shape == (33,)


def test_online_stats_checkpoint_round_trip(nk):
    rng = np.random.default_rng(3)
    est = nk.stats.online_statistics(rng.standard_normal((32, 20)), max_lag=16)
    blob = nk.serialization.dict_to_bytes(est.state_dict())
    back = nk.stats.OnlineStats.from_state_dict(nk.serialization.dict_from_bytes(blob))
    nxt = rng.standard_normal((32, 7))
    a, b = est.update(nxt), back.update(nxt)
    for k in KEYS:
        assert torch.equal(a._s[k], b._s[k])
    assert a.get_stats().as_array().tolist() == b.get_stats().as_array().tolist()
