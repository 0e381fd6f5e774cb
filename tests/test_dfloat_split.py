"""The float64 -> (hi, lo) float32 split of the double-float sweeps
(tdscha_gb300/csrc/dfloat.cuh, split_f64), restated on the bit pattern in
numpy: the claimed bounds hold over values spanning 70 decades.  The CUDA
function computes the same integer expressions (exponent rebiased by 896, low
29 mantissa bits as an integer scaled by 2^(exponent - 52))."""
import numpy as np


def split_f64(x):
    b = np.asarray(x, dtype=np.float64).view(np.uint64)
    hw = (b >> np.uint64(32)).astype(np.uint64)
    lw = (b & np.uint64(0xffffffff)).astype(np.uint64)
    e = (hw >> np.uint64(20)) & np.uint64(0x7ff)
    fs = ((hw << np.uint64(3)) | (lw >> np.uint64(29))) & np.uint64(0xffffffff)
    hb = (((fs - np.uint64(0xC0000000)) & np.uint64(0xffffffff)) & np.uint64(0x7fffffff)) | (
        hw & np.uint64(0x80000000))
    scale_bits = ((hb & np.uint64(0xff800000)) - np.uint64(52 << 23)) & np.uint64(0xffffffff)
    with np.errstate(over="ignore", invalid="ignore"):
        scale = scale_bits.astype(np.uint32).view(np.float32)
        lo = (lw & np.uint64(0x1fffffff)).astype(np.float32) * scale
    hi = np.where(e > 896, hb.astype(np.uint32).view(np.float32), np.float32(0))
    lo = np.where(e > 948, lo, np.float32(0))
    return hi, lo


def test_split_bounds():
    rng = np.random.default_rng(0)
    x = rng.standard_normal(200000) * 10.0 ** rng.uniform(-40, 30, 200000)
    x = np.concatenate([x, [0.0, -0.0, 1.0, -1.0, 2.0 ** -126, 2.0 ** -74, 2.0 ** -73, 1e-300,
                            5e-324, 3.0e38, -2.5e-7]])
    hi, lo = split_f64(x)
    rec = hi.astype(np.float64) + lo.astype(np.float64)
    big = np.abs(x) >= 2.0 ** -74
    rel = np.abs(rec - x)[big] / np.abs(x[big])
    assert rel.max() <= 2.0 ** -48
    # hi is x truncated: |hi| <= |x|, same sign; |lo| <= 2^-23 |hi|
    assert np.all(np.abs(hi[big].astype(np.float64)) <= np.abs(x[big]))
    assert np.all(np.sign(hi[big]) == np.sign(x[big]))
    assert np.all(np.abs(lo[big]) <= 2.0 ** -23 * np.abs(hi[big]))
    # 2^-126 <= |x| < 2^-74: lo dropped, error below 2^-97
    mid = (np.abs(x) < 2.0 ** -74) & (np.abs(x) >= 2.0 ** -126)
    assert np.abs(rec - x)[mid].max() <= 2.0 ** -97
    # |x| < 2^-126, zero included: both parts zero
    tiny = np.abs(x) < 2.0 ** -126
    assert np.all(rec[tiny] == 0)


def test_split_products_bound():
    """A double-float product with the hi*hi rounding error and both cross
    terms (df_fma_acc) agrees with the float64 product to about 2^-45.5: the
    dropped lo*lo term is at most 2^-46 of the product, each split adds
    2^-48."""
    rng = np.random.default_rng(1)
    a = rng.standard_normal(50000)
    b = rng.standard_normal(50000)
    ah, al = split_f64(a)
    bh, bl = split_f64(b)
    ah64, al64, bh64, bl64 = (v.astype(np.float64) for v in (ah, al, bh, bl))
    # hi*hi exactly (a float32 product fits in float64), cross terms, lo*lo dropped
    prod = ah64 * bh64 + (ah64 * bl64 + al64 * bh64)
    rel = np.abs(prod - a * b) / np.abs(a * b)
    assert rel.max() <= 1.5 * 2.0 ** -46 + 2 * 2.0 ** -48
