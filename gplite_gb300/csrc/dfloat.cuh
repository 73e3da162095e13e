// Double-float arithmetic: a value held as two FP32 numbers whose sum it is
// (Dekker, "A floating-point technique for extending the available precision",
// Numer. Math. 18, 1971; Knuth, TAOCP vol. 2, 4.2.2), and conversions between
// doubles and such pairs that use integer instructions only, for kernels where
// the FP64 pipe of this part (about 2 lane operations per clock per SM, against
// 128 for FP32) is the scarce unit. Operations carry ~2^-44 of their operands'
// size; the conversions are exact up to the pair's 48 significand bits.
#pragma once
#include <stdint.h>

namespace gpgp {

struct __align__(8) f2 {  // 8-byte aligned: one 64-bit shared-memory access per pair
  float h, l;
};

// s + e = a + b exactly
__device__ __forceinline__ f2 f2_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  return f2{s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
// s + e = a + b exactly, for |a| >= |b| (or a = 0)
__device__ __forceinline__ f2 f2_fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return f2{s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ f2 f2_neg(f2 a) { return f2{-a.h, -a.l}; }
__device__ __forceinline__ f2 f2_mul(f2 a, f2 b) {
  const float p = __fmul_rn(a.h, b.h);
  float e = __fmaf_rn(a.h, b.h, -p);  // TwoProd: p + e = a.h b.h exactly
  e = __fmaf_rn(a.h, b.l, e);
  e = __fmaf_rn(a.l, b.h, e);
  return f2_fast_two_sum(p, e);
}
// a + b c
__device__ __forceinline__ f2 f2_fma(f2 b, f2 c, f2 a) {
  const float p = __fmul_rn(b.h, c.h);
  float pe = __fmaf_rn(b.h, c.h, -p);
  pe = __fmaf_rn(b.h, c.l, pe);
  pe = __fmaf_rn(b.l, c.h, pe);
  const f2 s = f2_two_sum(a.h, p);
  return f2_fast_two_sum(s.h, __fadd_rn(s.l, __fadd_rn(a.l, pe)));
}
// 1 / sqrt(d) for d.h a normal positive FP32 number: the FP32 estimate and one
// Newton step x (1 + r / 2), r = 1 - d x^2 formed from exact products (the
// estimate's 2^-22 becomes ~2^-43)
__device__ __forceinline__ f2 f2_rsqrt(f2 d) {
  const float x = rsqrtf(d.h);
  const float y = __fmul_rn(x, x);
  const f2 m = f2_mul(d, f2{y, __fmaf_rn(x, x, -y)});
  const float r = __fsub_rn(__fsub_rn(1.0f, m.h), m.l);  // 1 - m.h is exact (Sterbenz)
  return f2_fast_two_sum(x, __fmul_rn(__fmul_rn(0.5f, x), r));
}


// (hi, lo) with hi + lo = a to 2^-48 relative, from a's bits: hi takes the top 24
// significand bits (truncated, so |lo| < ulp(hi)), lo the next 29 rounded to 24.
// Zero returns (+-0, 0); values whose lo would leave the FP32 normal range
// (|a| < 2^-74 or |a| >= 2^128, NaN, Inf) take FP64 conversions out of line.
static __device__ __noinline__ f2 f2_of_slow(double a) {
  const float h = __double2float_rn(a);
  return f2{h, __double2float_rn(a - (double)h)};
}
__device__ __forceinline__ f2 f2_of(double a) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(a);
  const unsigned sg = (unsigned)(b >> 32) & 0x80000000u;
  if ((b << 1) == 0ull) return f2{__uint_as_float(sg), 0.0f};
  const int ef = (int)((b >> 52) & 0x7FFull) - 1023 + 127;  // FP32 exponent field of a
  if (ef < 53 || ef > 254) return f2_of_slow(a);
  const unsigned hb = sg | ((unsigned)ef << 23) | (unsigned)((b >> 29) & 0x7FFFFFull);
  const unsigned r = (unsigned)(b & 0x1FFFFFFFull);  // the low 29 significand bits, units of 2^(e-52)
  const float lo = __fmul_rn(__uint2float_rn(r), __uint_as_float((unsigned)(ef - 52) << 23));
  return f2{__uint_as_float(hb), __uint_as_float(__float_as_uint(lo) | sg)};
}

// (double)f * 2^sh, exact, by moving the float's fields into a double: the
// float exponent is rebiased and sh added; zero and out-of-range cases take ldexp
// out of line so that the common path is never if-converted into FP64 work
static __device__ __noinline__ double f2d_scaled_slow(float f, int sh) { return ldexp((double)f, sh); }

__device__ __forceinline__ double f2d_scaled(float f, int sh) {
  const uint32_t b = __float_as_uint(f);
  if ((b << 1) == 0u) return 0.0;
  const uint32_t ef = (b >> 23) & 0xFFu;
  const int ed = (int)ef - 127 + 1023 + sh;
  if (ef == 0u || ef == 0xFFu || ed <= 0 || ed >= 2047) return f2d_scaled_slow(f, sh);
  const unsigned long long db = ((unsigned long long)(b >> 31) << 63) |
                                ((unsigned long long)ed << 52) |
                                ((unsigned long long)(b & 0x7FFFFFu) << 29);
  return __longlong_as_double((long long)db);
}

static __device__ __noinline__ double df2d_scaled_slow(float hi, float lo, int sh) {
  return f2d_scaled_slow(hi, sh) + f2d_scaled_slow(lo, sh);
}

// (hi + lo) 2^sh as a double without FP64 instructions. The pair is first
// renormalised (TwoSum), so |lo| <= ulp_float(hi) / 2 = 2^28 units in the last
// place of hi's double. hi's double has its low 29 mantissa bits clear, so lo,
// counted in those units, is added to or subtracted from the bit pattern of |hi|
// directly; a subtraction below a power of two lands in the binade beneath, whose
// unit is half as large, and takes twice the count. lo bits below the double's
// last place are dropped (an error under one unit). Zero, subnormal and
// out-of-range cases go to the FP64 path out of line.
__device__ __forceinline__ double df2d_scaled(float hi, float lo, int sh) {
  {
    const float s = __fadd_rn(hi, lo);
    const float bp = __fsub_rn(s, hi);
    lo = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bp)), __fsub_rn(lo, bp));
    hi = s;
  }
  const uint32_t bh = __float_as_uint(hi), bl = __float_as_uint(lo);
  // a zero sum (hi = 0 forces lo = 0 after TwoSum): common in zero-padded and
  // triangular operands, so it stays off the slow path
  if ((bh << 1) == 0u) return 0.0;
  const uint32_t eh = (bh >> 23) & 0xFFu, el = (bl >> 23) & 0xFFu;
  const int ed = (int)eh - 127 + 1023 + sh;
  const int shift = (int)el - (int)eh + 29;
  if (eh == 0u || eh == 0xFFu || el == 0xFFu || ed <= 1 || ed >= 2047 || shift > 5)
    return df2d_scaled_slow(hi, lo, sh);
  const uint32_t mh = bh & 0x7FFFFFu;
  uint32_t k = 0u;
  if (el != 0u) {
    const uint32_t ml = (bl & 0x7FFFFFu) | 0x800000u;
    k = shift >= 0 ? (ml << shift) : (shift > -24 ? (ml >> -shift) : 0u);
  }
  const bool opposite = ((bh ^ bl) >> 31) != 0u;
  if (opposite && mh == 0u) k <<= 1;
  unsigned long long mag = ((unsigned long long)ed << 52) | ((unsigned long long)mh << 29);
  mag = opposite ? mag - k : mag + k;
  return __longlong_as_double((long long)(mag | ((unsigned long long)(bh >> 31) << 63)));
}

__device__ __forceinline__ double f2_to_double(f2 a) { return df2d_scaled(a.h, a.l, 0); }

}  // namespace gpgp
