// FP64 elementary functions for the kernels bound by the FP64 pipe on this part
// (about 2 lane operations per clock per SM): each takes fewer FP64 instructions
// than the general library routine, at an error of about one ulp, and sends
// arguments outside its range to the library routine.
#pragma once
#include <math.h>
#include <stdint.h>

namespace gpgp {

static __device__ __noinline__ double rsqrt_slow(double x) { return 1.0 / sqrt(x); }

// 1/sqrt(x) for a positive finite x. The FP32 estimate rsqrtf(x) comes from a
// float built out of x's bits with integer operations (and goes back the same
// way), so no FP64 conversion or compare sits on the dependency chain; the
// estimate y0 (relative error ~2^-22) is refined by the binomial series
//   (1 - e)^(-1/2) = 1 + e/2 + 3e^2/8 + O(e^3),  e = 1 - x y0^2,
// four dependent FP64 operations whose neglected terms are ~2^-66. Arguments
// outside the float range take sqrt and division out of line.
__device__ __forceinline__ double rsqrt_fast(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const int E = (int)(b >> 52);
  if (E < 1023 - 125 || E > 1023 + 125) return rsqrt_slow(x);
  const float xf = __uint_as_float(((uint32_t)(E - 1023 + 127) << 23) | (uint32_t)((b >> 29) & 0x7FFFFFu));
  const uint32_t yb = __float_as_uint(rsqrtf(xf));
  const double y0 = __longlong_as_double(
      (long long)(((unsigned long long)(((yb >> 23) & 0xFFu) - 127u + 1023u) << 52) |
                  ((unsigned long long)(yb & 0x7FFFFFu) << 29)));
  const double e = fma(-(x * y0), y0, 1.0);
  return fma(y0 * e, fma(e, 0.375, 0.5), y0);
}

static __device__ __noinline__ double sqrt_slow(double x) { return sqrt(x); }

// sqrt(x) = x (1/sqrt(x)) for x in [2^-125, 2^126); zero, other magnitudes and
// non-finite arguments go to the library sqrt.
__device__ __forceinline__ double sqrt_fast(double x) {
  const int E = (int)((unsigned long long)__double_as_longlong(x) >> 52);
  if (E < 1023 - 125 || E > 1023 + 125) return sqrt_slow(x);
  return x * rsqrt_fast(x);
}

// 2^(j/64), j = 0..63, each the double nearest to the exact value
static __device__ const double kExp2Tab[64] = {
    0x1.0000000000000p+0, 0x1.02c9a3e778061p+0, 0x1.059b0d3158574p+0, 0x1.0874518759bc8p+0,
    0x1.0b5586cf9890fp+0, 0x1.0e3ec32d3d1a2p+0, 0x1.11301d0125b51p+0, 0x1.1429aaea92de0p+0,
    0x1.172b83c7d517bp+0, 0x1.1a35beb6fcb75p+0, 0x1.1d4873168b9aap+0, 0x1.2063b88628cd6p+0,
    0x1.2387a6e756238p+0, 0x1.26b4565e27cddp+0, 0x1.29e9df51fdee1p+0, 0x1.2d285a6e4030bp+0,
    0x1.306fe0a31b715p+0, 0x1.33c08b26416ffp+0, 0x1.371a7373aa9cbp+0, 0x1.3a7db34e59ff7p+0,
    0x1.3dea64c123422p+0, 0x1.4160a21f72e2ap+0, 0x1.44e086061892dp+0, 0x1.486a2b5c13cd0p+0,
    0x1.4bfdad5362a27p+0, 0x1.4f9b2769d2ca7p+0, 0x1.5342b569d4f82p+0, 0x1.56f4736b527dap+0,
    0x1.5ab07dd485429p+0, 0x1.5e76f15ad2148p+0, 0x1.6247eb03a5585p+0, 0x1.6623882552225p+0,
    0x1.6a09e667f3bcdp+0, 0x1.6dfb23c651a2fp+0, 0x1.71f75e8ec5f74p+0, 0x1.75feb564267c9p+0,
    0x1.7a11473eb0187p+0, 0x1.7e2f336cf4e62p+0, 0x1.82589994cce13p+0, 0x1.868d99b4492edp+0,
    0x1.8ace5422aa0dbp+0, 0x1.8f1ae99157736p+0, 0x1.93737b0cdc5e5p+0, 0x1.97d829fde4e50p+0,
    0x1.9c49182a3f090p+0, 0x1.a0c667b5de565p+0, 0x1.a5503b23e255dp+0, 0x1.a9e6b5579fdbfp+0,
    0x1.ae89f995ad3adp+0, 0x1.b33a2b84f15fbp+0, 0x1.b7f76f2fb5e47p+0, 0x1.bcc1e904bc1d2p+0,
    0x1.c199bdd85529cp+0, 0x1.c67f12e57d14bp+0, 0x1.cb720dcef9069p+0, 0x1.d072d4a07897cp+0,
    0x1.d5818dcfba487p+0, 0x1.da9e603db3285p+0, 0x1.dfc97337b9b5fp+0, 0x1.e502ee78b3ff6p+0,
    0x1.ea4afa2a490dap+0, 0x1.efa1bee615a27p+0, 0x1.f50765b6e4540p+0, 0x1.fa7c1819e90d8p+0,
};

static __device__ __noinline__ double exp_slow(double x) { return exp(x); }

// e^x by the table-driven method of P. T. P. Tang (ACM TOMS 15(2), 1989):
// x = N ln2/64 + r with N = round(64 x / ln2) and |r| <= ln2/128, N = 64 m + j,
// e^x = 2^m 2^(j/64) e^r. e^r - 1 is its Taylor polynomial of degree 5 (the
// remainder is below 2^-54 relative on that range), 2^(j/64) comes from the
// table above, and m is added to the exponent field. The reduction subtracts
// N ln2/64 in two FMAs (ln2/64 as a leading double plus the double nearest to
// the rest). Arguments outside (-707, 709), where the result would be subnormal
// or infinite, and NaN go to the library exp.
__device__ __forceinline__ double exp_fast(double x) {
  if (!(x > -707.0 && x < 709.0)) return exp_slow(x);
  const double t = fma(x, 0x1.71547652b82fep+6, 0x1.8p52);  // 1.5 2^52 + N
  const int N = __double2loint(t);
  const double Nd = t - 0x1.8p52;
  double r = fma(-Nd, 0x1.62e42fefa39efp-7, x);
  r = fma(-Nd, 0x1.abc9e3b39803fp-62, r);
  double q = fma(r, 1.0 / 120.0, 1.0 / 24.0);
  q = fma(q, r, 1.0 / 6.0);
  q = fma(q, r, 0.5);
  q = fma(q, r, 1.0);
  const double p = q * r;
  const double T = __ldg(&kExp2Tab[N & 63]);
  const double y = fma(T, p, T);
  const int m = N >> 6;  // floor(N / 64)
  return __hiloint2double(__double2hiint(y) + (m << 20), __double2loint(y));
}

}  // namespace gpgp
