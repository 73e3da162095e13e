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
// a + b for pairs (the "sloppy" sum: ~2^-44 of the operands' size)
__device__ __forceinline__ f2 f2_add(f2 a, f2 b) {
  const f2 s = f2_two_sum(a.h, b.h);
  return f2_fast_two_sum(s.h, __fadd_rn(s.l, __fadd_rn(a.l, b.l)));
}
__device__ __forceinline__ f2 f2_scale2(f2 a, float p2) { return f2{__fmul_rn(a.h, p2), __fmul_rn(a.l, p2)}; }

// 2^(j/64), j = 0..63, as pairs: the FP32 number nearest to the exact value and the
// FP32 number nearest to the rest (generated from 80-digit decimal arithmetic)
static __device__ const float kExp2TabDF[64][2] = {
    {0x1.0000000000000p+0f, 0x0.0p+0f},
    {0x1.02c9a40000000p+0f, -0x1.887fa00000000p-28f},
    {0x1.059b0e0000000p+0f, -0x1.9d4f520000000p-25f},
    {0x1.0874520000000p+0f, -0x1.e2990e0000000p-26f},
    {0x1.0b55860000000p+0f, 0x1.9f31220000000p-25f},
    {0x1.0e3ec40000000p+0f, -0x1.a585cc0000000p-25f},
    {0x1.11301e0000000p+0f, -0x1.fdb4960000000p-25f},
    {0x1.1429aa0000000p+0f, 0x1.d525bc0000000p-25f},
    {0x1.172b840000000p+0f, -0x1.c157420000000p-27f},
    {0x1.1a35be0000000p+0f, 0x1.6df96e0000000p-25f},
    {0x1.1d48740000000p+0f, -0x1.d2e8ca0000000p-25f},
    {0x1.2063b80000000p+0f, 0x1.0c519a0000000p-25f},
    {0x1.2387a60000000p+0f, 0x1.ceac480000000p-25f},
    {0x1.26b4560000000p+0f, 0x1.789f380000000p-26f},
    {0x1.29e9e00000000p+0f, -0x1.5c04240000000p-25f},
    {0x1.2d285a0000000p+0f, 0x1.b900c20000000p-26f},
    {0x1.306fe00000000p+0f, 0x1.4636e20000000p-25f},
    {0x1.33c08c0000000p+0f, -0x1.b37d200000000p-25f},
    {0x1.371a740000000p+0f, -0x1.18aac60000000p-25f},
    {0x1.3a7db40000000p+0f, -0x1.634c020000000p-25f},
    {0x1.3dea640000000p+0f, 0x1.8246840000000p-25f},
    {0x1.4160a20000000p+0f, 0x1.f72e2a0000000p-28f},
    {0x1.44e0860000000p+0f, 0x1.8624b40000000p-30f},
    {0x1.486a2c0000000p+0f, -0x1.47d8660000000p-25f},
    {0x1.4bfdae0000000p+0f, -0x1.593abc0000000p-25f},
    {0x1.4f9b280000000p+0f, -0x1.2c5a6c0000000p-25f},
    {0x1.5342b60000000p+0f, -0x1.2c56100000000p-25f},
    {0x1.56f4740000000p+0f, -0x1.295b040000000p-25f},
    {0x1.5ab07e0000000p+0f, -0x1.5bd5ec0000000p-27f},
    {0x1.5e76f20000000p+0f, -0x1.4a5bd60000000p-25f},
    {0x1.6247ec0000000p+0f, -0x1.f8b5500000000p-25f},
    {0x1.6623880000000p+0f, 0x1.2a91120000000p-27f},
    {0x1.6a09e60000000p+0f, 0x1.9fcef40000000p-26f},
    {0x1.6dfb240000000p+0f, -0x1.cd72e80000000p-27f},
    {0x1.71f75e0000000p+0f, 0x1.1d8bee0000000p-25f},
    {0x1.75feb60000000p+0f, -0x1.37b3060000000p-25f},
    {0x1.7a11480000000p+0f, -0x1.829fd00000000p-25f},
    {0x1.7e2f340000000p+0f, -0x1.2616340000000p-25f},
    {0x1.82589a0000000p+0f, -0x1.accc7c0000000p-26f},
    {0x1.868d9a0000000p+0f, -0x1.2edb440000000p-26f},
    {0x1.8ace540000000p+0f, 0x1.15506e0000000p-27f},
    {0x1.8f1aea0000000p+0f, -0x1.baa2320000000p-26f},
    {0x1.93737c0000000p+0f, -0x1.e647440000000p-25f},
    {0x1.97d82a0000000p+0f, -0x1.0d8d840000000p-31f},
    {0x1.9c49180000000p+0f, 0x1.51f8480000000p-27f},
    {0x1.a0c6680000000p+0f, -0x1.2886a60000000p-26f},
    {0x1.a5503c0000000p+0f, -0x1.b83b540000000p-25f},
    {0x1.a9e6b60000000p+0f, -0x1.50c0480000000p-25f},
    {0x1.ae89fa0000000p+0f, -0x1.a94b140000000p-26f},
    {0x1.b33a2c0000000p+0f, -0x1.ec3a820000000p-26f},
    {0x1.b7f7700000000p+0f, -0x1.a094380000000p-25f},
    {0x1.bcc1ea0000000p+0f, -0x1.f687c60000000p-25f},
    {0x1.c199be0000000p+0f, -0x1.3d56b20000000p-27f},
    {0x1.c67f120000000p+0f, 0x1.cafa2a0000000p-25f},
    {0x1.cb720e0000000p+0f, -0x1.8837cc0000000p-27f},
    {0x1.d072d40000000p+0f, 0x1.40f1300000000p-25f},
    {0x1.d5818e0000000p+0f, -0x1.822dbc0000000p-27f},
    {0x1.da9e600000000p+0f, 0x1.ed99420000000p-27f},
    {0x1.dfc9740000000p+0f, -0x1.908c940000000p-25f},
    {0x1.e502ee0000000p+0f, 0x1.e2cffe0000000p-26f},
    {0x1.ea4afa0000000p+0f, 0x1.52486c0000000p-27f},
    {0x1.efa1be0000000p+0f, 0x1.cc2b440000000p-25f},
    {0x1.f507660000000p+0f, -0x1.246eb00000000p-26f},
    {0x1.fa7c180000000p+0f, 0x1.9e90d80000000p-28f}
};

// e^x for a pair x <= 0, by the table-driven method of P. T. P. Tang (ACM TOMS
// 15(2), 1989) in pair arithmetic: N = round(64 x / ln2) = 64 m + j, r = x - N ln2/64
// (|r| <= ln2/128) with ln2/64 = C1 + C2 + C3 (C1 of 9 significant bits, so that N C1
// and x - N C1 are exact; N C2 as an exact pair by an FMA), e^r - 1 = r + r^2/2 +
// r^2/2 v, v = r/3 (1 + r/4 (1 + r/5)) in FP32 (its rounding reaches the result at
// ~2^-50; the dropped terms r^6/720 are below 2^-56), and e^x = 2^m 2^(j/64) e^r.
// Relative error ~1e-15 for x >= -70 (checked against 50-digit decimal arithmetic
// in an FP32 emulation); below that the pair's low part leaves the FP32 normal
// range and the error grows towards 4e-11 relative (under 1e-45 absolute) at -80.
// x < -80 returns 0; NaN returns NaN.
__device__ __forceinline__ f2 f2_exp_neg(f2 x) {
  if (x.h < -80.0f) return f2{0.0f, 0.0f};
  const float t = __fmaf_rn(x.h, 0x1.715476p+6f, 0x1.8p+23f);  // 1.5 2^23 + N
  const int N = __float_as_int(t) - 0x4B400000;
  const float Nf = __fsub_rn(t, 0x1.8p+23f);
  const float rh = __fmaf_rn(-Nf, 0x1.63p-7f, x.h);  // exact
  const float p2 = __fmul_rn(Nf, -0x1.bd0106p-19f);
  const float e2 = __fmaf_rn(Nf, -0x1.bd0106p-19f, -p2);  // N C2 = p2 + e2 exactly
  f2 r = f2_two_sum(rh, -p2);
  r = f2_fast_two_sum(r.h, __fadd_rn(__fsub_rn(r.l, e2), __fmaf_rn(-Nf, 0x1.cf79acp-46f, x.l)));
  float v = __fmaf_rn(r.h, 0.2f, 1.0f);
  v = __fmaf_rn(__fmul_rn(r.h, 0.25f), v, 1.0f);
  v = __fmul_rn(__fmul_rn(r.h, 0x1.555556p-2f), v);  // u - 1
  const f2 r2 = f2_mul(r, r);
  const f2 h2 = f2{0.5f * r2.h, 0.5f * r2.l};
  const f2 em1 = f2_add(r, f2_add(h2, f2{__fmul_rn(h2.h, v), 0.0f}));
  const int j = N & 63, m = N >> 6;
  const f2 T = f2{kExp2TabDF[j][0], kExp2TabDF[j][1]};
  return f2_scale2(f2_fma(T, em1, T), __int_as_float((m + 127) << 23));
}

// sqrt(d) for a pair d >= 0 (A. H. Karp and P. Markstein, ACM TOMS 23(4), 1997):
// s0 = d x0 with x0 the FP32 estimate of 1/sqrt(d), then s0 + x0/2 (d - s0^2) with
// s0^2 as an exact pair; the error is about the square of the estimate's (~2^-44).
// d.h below 2^-100 returns 0.
__device__ __forceinline__ f2 f2_sqrt(f2 d) {
  if (!(d.h >= 7.8886090522101181e-31f)) return f2{0.0f, 0.0f};
  const float x0 = rsqrtf(d.h);
  const float s0 = __fmul_rn(d.h, x0);
  const float p = __fmul_rn(s0, s0);
  const float pe = __fmaf_rn(s0, s0, -p);
  const float res = __fadd_rn(__fsub_rn(__fsub_rn(d.h, p), pe), d.l);
  return f2_fast_two_sum(s0, __fmul_rn(__fmul_rn(0.5f, x0), res));
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
