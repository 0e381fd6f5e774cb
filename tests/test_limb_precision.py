"""Operand precision of the tensor-core limb formats, emulated on the CPU.

The mixed path feeds tcgen05.mma kind::f16 with two fp16 limbs per operand,
x = hi + 2^-11 lo with hi = fp16(x), lo = fp16((x - hi) 2^11) after a per-row
scale into [-1, 1] (split_f16 in tdscha_gb300/csrc/perturb_mixed.cu), and
forms hi*hi + hi*lo + lo*hi.  These tests restate that split in numpy and
compare it, on the same operands, with the other formats a contraction could
use: two bf16 limbs (the first version of the path), one tf32 limb, and two
tf32 limbs (kind::tf32, half the dense rate of kind::f16 and twice the operand
bytes).  Products are accumulated in float64 here so that only the operand
rounding is measured.
"""
import numpy as np


def _round_mantissa(x, keep):
    """float32 x rounded to `keep` explicit mantissa bits, nearest even."""
    b = np.asarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    drop = 23 - keep
    b = (b + (1 << (drop - 1)) - 1 + ((b >> drop) & 1)) >> drop << drop
    return b.astype(np.uint32).view(np.float32).astype(np.float64)


def _tf32(x):
    return _round_mantissa(x, 10)


def _bf16(x):
    return _round_mantissa(x, 7)


def _limbs_f16(x):
    x = np.asarray(x, dtype=np.float32)
    hi = x.astype(np.float16)
    lo = ((x - hi.astype(np.float32)) * np.float32(2048.0)).astype(np.float16)
    return hi.astype(np.float64), lo.astype(np.float64) * 2.0 ** -11


def _limbs(x, rnd):
    x = np.asarray(x, dtype=np.float32)
    hi = rnd(x)
    lo = rnd((x.astype(np.float64) - hi).astype(np.float32))
    return hi, lo


def _three_products(a, b):
    return a[0] * b[0] + a[0] * b[1] + a[1] * b[0]


def _operands(seed, n, decades):
    """Scaled operands: |x| <= 1 spread over `decades` powers of two, as the
    per-mode scaling leaves the ensemble displacements and the Y1 rows."""
    rng = np.random.default_rng(seed)
    x = rng.uniform(-1, 1, n) * 2.0 ** -rng.uniform(0, decades, n)
    y = rng.uniform(-1, 1, n) * 2.0 ** -rng.uniform(0, decades, n)
    return x.astype(np.float32), y.astype(np.float32)


def _errors(seed=0, n=1 << 15, decades=8):
    x, y = _operands(seed, n, decades)
    exact = x.astype(np.float64) * y.astype(np.float64)
    formats = {
        "f16x3": _three_products(_limbs_f16(x), _limbs_f16(y)),
        "tf32x3": _three_products(_limbs(x, _tf32), _limbs(y, _tf32)),
        "bf16x3": _three_products(_limbs(x, _bf16), _limbs(y, _bf16)),
        "tf32x1": _tf32(x) * _tf32(y),
    }
    out = {}
    for k, p in formats.items():
        # per product against the scale the rows were normalised to (1 x 1),
        # and for a dot product of n terms against sum |x y|
        out[k] = (np.max(np.abs(p - exact)), abs((p - exact).sum()) / np.abs(exact).sum())
    return out


def test_f16_limbs_carry_22_bits_at_the_scale():
    e = _errors()
    # hi*hi + hi*lo + lo*hi with 11-bit limbs: the dropped lo*lo and the lo
    # rounding leave ~2^-22 of |x||y| for full-scale operands
    assert e["f16x3"][0] <= 2.0 ** -21
    assert e["tf32x3"][0] <= 2.0 ** -21


def test_f16_and_tf32_limbs_agree_in_dot_products():
    for seed in range(3):
        e = _errors(seed)
        assert e["f16x3"][1] <= 1e-8
        assert e["tf32x3"][1] <= 1e-8
        assert e["f16x3"][1] <= 1.01 * e["tf32x3"][1] + 1e-12


def test_bf16_limbs_and_single_tf32_fall_short():
    e = _errors()
    # 8-bit limbs (16 bits in all) and one 11-bit tf32 operand lose 2^6 and
    # 2^11 against the fp16 pair
    assert e["bf16x3"][1] >= 30 * e["f16x3"][1]
    assert e["tf32x1"][1] >= 1000 * e["f16x3"][1]
    assert e["tf32x1"][0] >= 2.0 ** -13


def test_f16_limbs_error_bound_over_the_scaled_range():
    # |x - hi - 2^-11 lo| <= 2^-22 |x| + 2^-36 for every |x| <= 1: the low limb
    # is lifted by 2^11, so it reaches the fp16 subnormal spacing (2^-24) only
    # for |x| below ~2^-14, where the absolute error stays under 2^-36
    rng = np.random.default_rng(5)
    x = (rng.choice([-1.0, 1.0], 1 << 16) * 2.0 ** -rng.uniform(0, 30, 1 << 16)).astype(np.float32)
    hi, lo = _limbs_f16(x)
    xd = x.astype(np.float64)
    assert np.all(np.abs(hi + lo - xd) <= 2.0 ** -22 * np.abs(xd) + 2.0 ** -36)
    big = np.abs(xd) >= 2.0 ** -14
    assert np.max(np.abs(hi + lo - xd)[big] / np.abs(xd[big])) <= 2.0 ** -22
