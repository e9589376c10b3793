"""The arithmetic the mode-4 Gram rests on, modelled in numpy FP32 / FP16 (no
GPU): c = t - s0 (|c| < 2) rounded to a multiple of 2^-19 splits into FP16 hi =
rint(256 c), |hi| <= 512, and lo = rint((256 c - hi) 2^11) 2^-11, both exact in
FP16, with (hi + lo) / 256 == c exactly; a 64-wide slab of hi * hi' products is
an integer of at most 2^24, exact in FP32 however it is summed.  (The kernels:
gram_shift_kernel with terms = 3, gram_split_fixed_kernel.)"""
import numpy as np


def _grid(c):
    c = np.asarray(c, dtype=np.float32)
    return (np.rint(c * np.float32(524288.0)) / np.float32(524288.0)).astype(np.float32)


def _split(c):
    u = (c * np.float32(256.0)).astype(np.float32)
    hi = np.rint(u).astype(np.float32)
    lo = (np.rint((u - hi) * np.float32(2048.0)) * np.float32(1.0 / 2048.0)).astype(np.float32)
    return hi, lo


def test_split_is_exact_in_fp16():
    rng = np.random.default_rng(0)
    t = np.tanh(rng.normal(scale=2.0, size=200000)).astype(np.float32)
    s0 = np.float32(t.mean())
    c = _grid((t - s0).astype(np.float32))
    edges = _grid(np.array([1.9999999, -1.9999999, 2.0 - 2 ** -19, 0.0, 2 ** -19, -2 ** -20],
                           dtype=np.float32))
    for cc in (c, edges):
        hi, lo = _split(cc)
        assert np.abs(hi).max() <= 512
        assert np.array_equal(hi.astype(np.float16).astype(np.float32), hi)
        assert np.array_equal(lo.astype(np.float16).astype(np.float32), lo)
        assert np.array_equal(((hi.astype(np.float64) + lo) / 256.0), cc.astype(np.float64))


def test_slab_sums_of_hi_products_are_exact():
    rng = np.random.default_rng(1)
    hi = np.rint(rng.uniform(-512, 512, size=(64, 1000))).astype(np.float32)
    hi[:, :4] = 512.0  # the largest slab: 64 * 512^2 = 2^24
    hi[:, 4:8] = -512.0
    exact = (hi.astype(np.int64)[:, :, None] * hi.astype(np.int64)[:, None, :8]).sum(axis=0)
    assert np.abs(exact).max() <= 2 ** 24
    # any summation order in FP32 gives the integer exactly
    p = hi[:, :, None] * hi[:, None, :8]
    fwd = np.zeros(p.shape[1:], dtype=np.float32)
    for k in range(64):
        fwd = (fwd + p[k]).astype(np.float32)
    rev = np.zeros(p.shape[1:], dtype=np.float32)
    for k in range(63, -1, -1):
        rev = (rev + p[k]).astype(np.float32)
    assert np.array_equal(fwd.astype(np.int64), exact)
    assert np.array_equal(rev.astype(np.int64), exact)
