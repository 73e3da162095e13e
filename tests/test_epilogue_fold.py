"""The sliced GEMM's epilogue turns a double-float pair (hi, lo) into a double
with integer operations (df2d_scaled in gplite_gb300/csrc/mixed.cu): TwoSum
renormalisation, then lo counted in units of the last place of hi's double and
added to its bit pattern, with a borrow below a power of two taking twice the
count. This restates that function bit for bit in NumPy (IEEE float32 round to
nearest, as __fadd_rn) and checks it against exact rational arithmetic: within
one unit in the last place of the double, and exactly 0 for a zero sum. The
device code itself is covered by the GPU parity tests."""
from fractions import Fraction

import numpy as np


def _b32(x):
    return int(np.array(x, dtype=np.float32).view(np.uint32))


def fold(hi, lo, sh):
    hi, lo = np.float32(hi), np.float32(lo)
    s = np.float32(hi + lo)
    bp = np.float32(s - hi)
    lo = np.float32(np.float32(hi - np.float32(s - bp)) + np.float32(lo - bp))
    hi = s
    bh, bl = _b32(hi), _b32(lo)
    if (bh << 1) & 0xFFFFFFFF == 0:
        return 0.0
    eh, el = (bh >> 23) & 0xFF, (bl >> 23) & 0xFF
    ed = eh - 127 + 1023 + sh
    shift = el - eh + 29
    if eh == 0 or eh == 0xFF or el == 0xFF or ed <= 1 or ed >= 2047 or shift > 5:
        return float(np.ldexp(np.float64(hi), sh) + np.ldexp(np.float64(lo), sh))
    mh = bh & 0x7FFFFF
    k = 0
    if el != 0:
        ml = (bl & 0x7FFFFF) | 0x800000
        k = (ml << shift) if shift >= 0 else ((ml >> -shift) if shift > -24 else 0)
    opposite = ((bh ^ bl) >> 31) != 0
    if opposite and mh == 0:
        k <<= 1
    mag = (ed << 52) | (mh << 29)
    mag = mag - k if opposite else mag + k
    return np.array(mag | ((bh >> 31) << 63), dtype=np.uint64).view(np.float64).item()


def test_fold_is_within_one_ulp_of_the_exact_sum():
    rng = np.random.default_rng(0)
    worst = 0.0
    for i in range(20000):
        mode, e = i % 5, int(rng.integers(-40, 40))
        if mode == 0:  # a renormalised pair
            hi = rng.standard_normal() * 2.0 ** e
            lo = rng.standard_normal() * 2.0 ** (e - 30)
        elif mode == 1:  # hi a power of two, lo of the other sign: borrow into the binade beneath
            hi = 2.0 ** e * (1 if rng.uniform() < 0.5 else -1)
            lo = -np.sign(hi) * rng.uniform(0, 1) * 2.0 ** (e - 24)
        elif mode == 2:  # lo above half an ulp of hi (renormalised first)
            hi = rng.standard_normal() * 2.0 ** e
            lo = rng.standard_normal() * 2.0 ** (e - 20)
        elif mode == 3:  # exact cancellation
            hi = np.float32(rng.standard_normal() * 2.0 ** e)
            lo = -hi
        else:  # zeros
            hi = 0.0 if rng.uniform() < 0.5 else rng.standard_normal()
            lo = 0.0
        hi, lo, sh = np.float32(hi), np.float32(lo), int(rng.integers(-60, 60))
        got = fold(hi, lo, sh)
        exact = (Fraction(float(hi)) + Fraction(float(lo))) * Fraction(2) ** sh
        if exact == 0:
            assert got == 0.0
            continue
        worst = max(worst, float(abs((Fraction(got) - exact) / exact)))
    assert worst <= 2.0 ** -52
