"""Bit-level conversions of the pair-arithmetic kernels, restated with NumPy integer operations and
checked against their claims: the double -> float-pair split (vh_df.cuh df_split), the exact
float -> double widening (f2d_exact) and the float-reciprocal integer division of the front kernel
(vh_chol.cu div_small).  The device code performs the same bit operations."""
import numpy as np


def split_pair(d):
    """df_split: hi = sign, exponent and top 23 fraction bits of d (truncated); lo = the remaining 29
    fraction bits rounded to a float.  Only the fast range 949 <= biased exponent <= 1150."""
    b = d.view(np.uint64)
    hw = (b >> np.uint64(32)).astype(np.uint32)
    lw = (b & np.uint64(0xFFFFFFFF)).astype(np.uint32)
    e = (hw >> 20) & 0x7FF
    fast = (e >= 949) & (e <= 1150)
    s = hw & np.uint32(0x80000000)
    ef = np.where(fast, e - 896, 1).astype(np.uint32)
    hi = (s | (ef << 23) | ((hw & 0xFFFFF) << 3) | (lw >> 29)).view(np.float32)
    scale = (np.where(fast, e - 948, 1).astype(np.uint32) << 23).view(np.float32)
    rem = (lw & 0x1FFFFFFF).astype(np.float32) * scale   # uint32 -> float rounds to nearest
    lo = (rem.view(np.uint32) | s).view(np.float32)
    return hi, lo, fast


def test_split_reconstructs_to_47_bits():
    rng = np.random.default_rng(7)
    mant = rng.uniform(1.0, 2.0, 400_000)
    expo = rng.integers(-70, 120, mant.size)
    sign = rng.choice([-1.0, 1.0], mant.size)
    d = sign * np.ldexp(mant, expo)
    hi, lo, fast = split_pair(d)
    assert fast.all()
    rec = hi.astype(np.float64) + lo.astype(np.float64)
    rel = np.abs(rec - d) / np.abs(d)
    assert rel.max() <= 2.0**-47
    # |lo| < ulp(hi): lo never reaches the weight of hi's last fraction bit
    ulp = np.abs(np.spacing(hi)).astype(np.float64)
    assert np.all(np.abs(lo.astype(np.float64)) < ulp)


def test_split_range_limits():
    # the fast path covers [2^-74, 2^127); outside it the device falls back to the conversion
    # instructions (and zero gives zero)
    d = np.array([2.0**-74, 2.0**127 * 1.999, 2.0**-75, 2.0**128, 0.0, 1.0])
    _, _, fast = split_pair(d)
    assert fast.tolist() == [True, True, False, False, False, True]


def test_float_to_double_widening_is_exact():
    rng = np.random.default_rng(3)
    u = rng.integers(0, 2**32, 1_000_000, dtype=np.uint64).astype(np.uint32)
    e = (u >> 23) & 0xFF
    u = u[(e >= 1) & (e <= 254)]            # normal floats: the integer path
    hw = (u & 0x80000000) | (((u >> 23) & 0xFF) + 896).astype(np.uint32) << 20 | ((u & 0x7FFFFF) >> 3)
    lw = (u & 7).astype(np.uint64) << np.uint64(29)
    d = ((hw.astype(np.uint64) << np.uint64(32)) | lw).view(np.float64)
    assert np.array_equal(d, u.view(np.float32).astype(np.float64))


def test_float_reciprocal_division_is_exact():
    # a / d for the front orders d <= 240 and every flat index a < d^2 of a front
    for d in range(1, 241):
        rd = np.float32(1.0) / np.float32(d)
        a = np.arange(d * d, dtype=np.int64)
        q = (a.astype(np.float32) * rd).astype(np.int64)
        q = np.where(q * d > a, q - 1, np.where((q + 1) * d <= a, q + 1, q))
        assert np.array_equal(q, a // d), d
