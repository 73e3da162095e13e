// Likelihood kernels: Laplace pseudo-data (R/lik.R:188-201, 372-454), EP site
// updates with Gauss-Hermite tilted moments (R/lik.R:207-270), log-likelihood
// sums (R/lik.R:301-366) and LOO predictive densities (R/gp_loo.R:90-96).
// One thread per observation; sums use fixed-order block reductions.
#include <math.h>

#include <algorithm>
#include <cmath>

#include "common.cuh"

namespace gpgp {

#define LN_SQRT_2PI 0.918938533204672741780329736406

__device__ __forceinline__ double response(const LikDev &L, double f) {
  if (L.kind == GPGP_LIK_POISSON) return exp(f);
  if (L.link == GPGP_LINK_PROBIT) return normcdf(f);
  return 1.0 / (1.0 + exp(-f));  // logit (R/lik.R:476-481)
}

__device__ __forceinline__ double xlogy(double x, double y) { return x == 0.0 ? 0.0 : x * log(y); }

// Digamma psi(x) for x > 0, from its recurrence psi(x) = psi(x + 1) - 1/x (lifting x
// to >= 12) and the asymptotic series psi(x) = ln x - 1/(2x) - sum_k B_2k / (2k x^2k)
// (Abramowitz & Stegun 6.3.18) through x^-14; the first omitted term is below
// 3e-18 at x = 12.
__device__ double digamma_pos(double x) {
  double acc = 0.0;
  while (x < 12.0) {
    acc -= 1.0 / x;
    x += 1.0;
  }
  const double r = 1.0 / x, r2 = r * r;
  // B_2k / (2k): 1/12, -1/120, 1/252, -1/240, 1/132, -691/32760, 1/12
  double p = 1.0 / 12.0;
  p = fma(p, r2, -691.0 / 32760.0);
  p = fma(p, r2, 1.0 / 132.0);
  p = fma(p, r2, -1.0 / 240.0);
  p = fma(p, r2, 1.0 / 252.0);
  p = fma(p, r2, -1.0 / 120.0);
  p = fma(p, r2, 1.0 / 12.0);
  return acc + (log(x) - 0.5 * r - r2 * p);
}

// log p(y | f) for one observation; f already includes the offset.
__device__ __forceinline__ double loglik1(const LikDev &L, double f, double y, double N) {
  switch (L.kind) {
    case GPGP_LIK_GAUSSIAN: {
      const double x = (y - f) / L.sigma;
      return -(LN_SQRT_2PI + 0.5 * x * x + log(L.sigma));  // stats::dnorm(log = TRUE)
    }
    case GPGP_LIK_BERNOULLI:
    case GPGP_LIK_BINOMIAL: {
      const double mu = response(L, f);
      const double lch = lgamma(N + 1.0) - lgamma(y + 1.0) - lgamma(N - y + 1.0);
      return lch + xlogy(y, mu) + xlogy(N - y, 1.0 - mu);
    }
    case GPGP_LIK_POISSON: {
      const double mu = exp(f);
      return xlogy(y, mu) - mu - lgamma(y + 1.0);
    }
    case GPGP_LIK_BETABINOM: {  // R/lik.R:332-354
      const double mu = response(L, f);
      const double a = mu / L.phi, b = (1.0 - mu) / L.phi;
      const double term1 = lgamma(N + 1.0) - lgamma(y + 1.0) - lgamma(N - y + 1.0);
      const double term2 = lgamma(y + a) + lgamma(N - y + b) - lgamma(N + a + b);
      const double term3 = lgamma(a + b) - lgamma(a) - lgamma(b);
      return term1 + term2 + term3;
    }
    default:
      return nan("");
  }
}

// d log p / d f (R/lik.R:372-443); f includes the offset.
__device__ __forceinline__ double loglik_d1(const LikDev &L, double f, double y, double N) {
  if (L.kind == GPGP_LIK_POISSON) {
    const double mu = exp(f);
    return (y / mu - 1.0) * mu;
  }
  const double mu = response(L, f);
  const double dmu =
      (L.link == GPGP_LINK_PROBIT) ? exp(-0.5 * f * f) * 0.398942280401432677939946059934 : mu * (1.0 - mu);
  if (L.kind == GPGP_LIK_BETABINOM) {  // R/lik.R:400-425
    const double a = mu / L.phi, b = (1.0 - mu) / L.phi;
    const double term2 = (dmu / L.phi) * (digamma_pos(y + a) - digamma_pos(N - y + b));
    const double term3 = (dmu / L.phi) * (-digamma_pos(a) + digamma_pos(b));
    return term2 + term3;
  }
  return dmu * (y / mu - (N - y) / (1.0 - mu));
}

__device__ __forceinline__ double trials_of(const LikDev &L, const double *trials, int64_t i) {
  if (L.kind == GPGP_LIK_BINOMIAL || L.kind == GPGP_LIK_BETABINOM) return trials[i];
  return 1.0;
}

// ---------------------------------------------------------------------------
__global__ void pseudodata_la_kernel(LikDev L, int64_t n, const double *__restrict__ f,
                                     const double *__restrict__ y,
                                     const double *__restrict__ trials,
                                     const double *__restrict__ offset, double *__restrict__ z,
                                     double *__restrict__ V) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (L.kind == GPGP_LIK_GAUSSIAN) {
    z[i] = y[i];
    V[i] = L.sigma * L.sigma;
    return;
  }
  const double eps = 1e-6;
  const double off = offset ? offset[i] : 0.0;
  const double N = trials_of(L, trials, i);
  const double fi = f[i];
  const double g = loglik_d1(L, fi + off, y[i], N);
  const double ge = loglik_d1(L, (fi + eps) + off, y[i], N);
  double g2 = (ge - g) / eps;  // forward difference (R/lik.R:449-454)
  const double sg = (g2 > 0.0) ? 1.0 : ((g2 < 0.0) ? -1.0 : 0.0);
  g2 = sg * fmax(fabs(g2), 1e-12);  // min_abs_curvature (R/lik.R:196-199)
  z[i] = fi - g / g2;
  V[i] = -1.0 / g2;
}

void lik_pseudodata_la(cudaStream_t s, const LikDev &lk, int64_t n, const double *f,
                       const double *y, const double *trials, const double *offset, double *z,
                       double *V) {
  if (n == 0) return;
  pseudodata_la_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(lk, n, f, y, trials, offset,
                                                                    z, V);
  GPGP_CHECK_LAUNCH();
}

// ---------------------------------------------------------------------------
__global__ void loglik_part_kernel(LikDev L, int64_t n, const double *__restrict__ f,
                                   const double *__restrict__ y,
                                   const double *__restrict__ trials,
                                   const double *__restrict__ offset, double *__restrict__ part) {
  __shared__ double red[256];
  double s = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * 256 + threadIdx.x; i < n; i += (int64_t)gridDim.x * 256) {
    const double off = offset ? offset[i] : 0.0;
    s += loglik1(L, f[i] + off, y[i], trials_of(L, trials, i));
  }
  red[threadIdx.x] = s;
  __syncthreads();
  for (int st = 128; st > 0; st >>= 1) {
    if (threadIdx.x < st) red[threadIdx.x] += red[threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

void lik_loglik(cudaStream_t s, const LikDev &lk, int64_t n, const double *f, const double *y,
                const double *trials, const double *offset, double *out_scalar, double *part) {
  const int nb = 64;  // part must hold 64 doubles
  loglik_part_kernel<<<nb, 256, 0, s>>>(lk, n, f, y, trials, offset, part);
  GPGP_CHECK_LAUNCH();
  sum_vec(s, part, nb, out_scalar);
}

// ---------------------------------------------------------------------------
constexpr int MAXQ = 64;

__global__ void ep_sites_kernel(LikDev L, int64_t n, int q, const double *__restrict__ ghx,
                                const double *__restrict__ ghw, const double *__restrict__ fmean,
                                const double *__restrict__ fvar, const double *__restrict__ z_old,
                                const double *__restrict__ P_old, const double *__restrict__ y,
                                const double *__restrict__ trials,
                                const double *__restrict__ offset, double damping,
                                double *__restrict__ z, double *__restrict__ V,
                                double *__restrict__ logC, double *__restrict__ cav_mean,
                                double *__restrict__ cav_var, int *__restrict__ flags) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double post_prec = 1.0 / fvar[i];
  const double post_mean = fmean[i];
  const double Po = P_old[i], zo = z_old[i];
  const double cp = post_prec - Po;
  const double cm = 1.0 / cp * (post_mean * post_prec - zo * Po);
  const double sd = sqrt(1.0 / cp);
  const double off = offset ? offset[i] : 0.0;
  const double N = trials_of(L, trials, i);
  double fg[MAXQ], ll[MAXQ], lk[MAXQ];
  bool nan_found = false;
  double mx = -INFINITY;
  for (int k = 0; k < q; ++k) {
    fg[k] = ghx[k] * sd + cm;
    ll[k] = loglik1(L, fg[k] + off, y[i], N);
    lk[k] = exp(ll[k]);
    if (isnan(lk[k])) {
      nan_found = true;
      lk[k] = 0.0;
      ll[k] = -INFINITY;
    }
    mx = fmax(mx, ll[k]);
  }
  double acc = 0.0;
  for (int k = 0; k < q; ++k) acc += ghw[k] * exp(ll[k] - mx);
  const double lC = mx + log(acc);
  const double C = exp(lC);
  double m1 = 0.0;
  for (int k = 0; k < q; ++k) m1 += fg[k] * lk[k] * ghw[k];
  const double mt = (1.0 / C) * m1;
  double m2 = 0.0;
  for (int k = 0; k < q; ++k) {
    const double dd = fg[k] - mt;
    m2 += dd * dd * lk[k] * ghw[k];
  }
  const double vt = (1.0 / C) * m2;
  const double vc = 1.0 / cp;
  double Pn = 1.0 / vt - 1.0 / vc;
  double nun = mt / vt - cm / vc;
  const double nuo = zo * Po;
  nun = damping * nun + (1.0 - damping) * nuo;
  Pn = damping * Pn + (1.0 - damping) * Po;
  const double zi = (1.0 / Pn) * nun;
  const double Vi = 1.0 / Pn;
  z[i] = zi;
  V[i] = Vi;
  logC[i] = lC;
  cav_mean[i] = cm;
  cav_var[i] = vc;
  int fl = 0;
  if (nan_found) fl |= 1;
  if (isnan(zi) || isnan(Vi)) fl |= 2;
  if (!(Vi > 0.0)) fl |= 4;
  if (fl) atomicOr(flags, fl);
}

void lik_ep_sites(cudaStream_t s, const LikDev &lk, int64_t n, int q, const double *ghx,
                  const double *ghw, const double *fmean, const double *fvar, const double *z_old,
                  const double *P_old, const double *y, const double *trials,
                  const double *offset, double damping, double *z, double *V, double *logC,
                  double *cav_mean, double *cav_var, int *flags) {
  if (n == 0) return;
  ep_sites_kernel<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(
      lk, n, q, ghx, ghw, fmean, fvar, z_old, P_old, y, trials, offset, damping, z, V, logC,
      cav_mean, cav_var, flags);
  GPGP_CHECK_LAUNCH();
}

// ---------------------------------------------------------------------------
__global__ void loo_gh_kernel(LikDev L, int64_t n, int q, const double *__restrict__ ghx,
                              const double *__restrict__ ghw, const double *__restrict__ mean,
                              const double *__restrict__ var, const double *__restrict__ y,
                              const double *__restrict__ trials,
                              const double *__restrict__ offset, double *__restrict__ loos) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double sd = sqrt(var[i]);
  const double off = offset ? offset[i] : 0.0;
  const double N = trials_of(L, trials, i);
  double ll[MAXQ];
  double mx = -INFINITY;
  for (int k = 0; k < q; ++k) {
    const double f = ghx[k] * sd + mean[i];
    ll[k] = loglik1(L, f + off, y[i], N);
    mx = fmax(mx, ll[k]);
  }
  double acc = 0.0;
  for (int k = 0; k < q; ++k) acc += ghw[k] * exp(ll[k] - mx);
  loos[i] = mx + log(acc);
}

void lik_loo_gh(cudaStream_t s, const LikDev &lk, int64_t n, int q, const double *ghx,
                const double *ghw, const double *mean, const double *var, const double *y,
                const double *trials, const double *offset, double *loos) {
  if (n == 0) return;
  loo_gh_kernel<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(lk, n, q, ghx, ghw, mean, var, y,
                                                            trials, offset, loos);
  GPGP_CHECK_LAUNCH();
}

// Monte Carlo LOO densities (R/gp_loo.R:97-103): per site, logsumexp over the draws of
// log p(y_i | mean_i + sd_i z_ik) minus log(draws); z is n x draws, column-major.
// One warp per site; the lanes share the draws, the maxima and sums are combined
// in a fixed order.
__global__ void loo_mc_kernel(LikDev L, int64_t n, int64_t draws, const double *__restrict__ z,
                              const double *__restrict__ mean, const double *__restrict__ var,
                              const double *__restrict__ y, const double *__restrict__ trials,
                              const double *__restrict__ offset, double *__restrict__ loos) {
  const int64_t i = (int64_t)blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  const int lane = threadIdx.x & 31;
  if (i >= n) return;
  const double sd = sqrt(var[i]);
  const double mu = mean[i];
  const double off = offset ? offset[i] : 0.0;
  const double N = trials_of(L, trials, i);
  const double yi = y[i];
  double mx = -INFINITY;
  for (int64_t k = lane; k < draws; k += 32) mx = fmax(mx, loglik1(L, (mu + sd * z[i + k * n]) + off, yi, N));
  for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  double acc = 0.0;
  for (int64_t k = lane; k < draws; k += 32)
    acc += exp(loglik1(L, (mu + sd * z[i + k * n]) + off, yi, N) - mx);
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane == 0) loos[i] = (mx + log(acc)) - log((double)draws);
}

void lik_loo_mc(cudaStream_t s, const LikDev &lk, int64_t n, int64_t draws, const double *z, const double *mean,
                const double *var, const double *y, const double *trials, const double *offset, double *loos) {
  if (n == 0) return;
  loo_mc_kernel<<<(unsigned)((n + 7) / 8), 256, 0, s>>>(lk, n, draws, z, mean, var, y, trials, offset, loos);
  GPGP_CHECK_LAUNCH();
}

// ---------------------------------------------------------------------------
// elementwise helpers
// ---------------------------------------------------------------------------
__global__ void axpby_kernel(int64_t n, double a, const double *__restrict__ x, double b,
                             double *__restrict__ y) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = a * x[i] + b * y[i];
}
void vec_axpby(cudaStream_t s, int64_t n, double a, const double *x, double b, double *y) {
  if (n == 0) return;
  axpby_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, a, x, b, y);
  GPGP_CHECK_LAUNCH();
}

__global__ void mul_kernel(int64_t n, const double *__restrict__ a, const double *__restrict__ b,
                           double *__restrict__ o) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) o[i] = a[i] * b[i];
}
void vec_mul(cudaStream_t s, int64_t n, const double *a, const double *b, double *out) {
  if (n == 0) return;
  mul_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, a, b, out);
  GPGP_CHECK_LAUNCH();
}

__global__ void rsqrt_kernel(int64_t n, const double *__restrict__ v, double *__restrict__ o) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) o[i] = sqrt(1.0 / v[i]);  // sqrt(1 / V) (R/laplace.R:27)
}
void vec_rsqrt(cudaStream_t s, int64_t n, const double *v, double *out) {
  if (n == 0) return;
  rsqrt_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, v, out);
  GPGP_CHECK_LAUNCH();
}

__global__ void dot_part_kernel(int64_t n, const double *__restrict__ a,
                                const double *__restrict__ b, double *__restrict__ part) {
  __shared__ double red[256];
  double s = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * 256 + threadIdx.x; i < n; i += (int64_t)gridDim.x * 256)
    s = fma(a[i], b[i], s);
  red[threadIdx.x] = s;
  __syncthreads();
  for (int st = 128; st > 0; st >>= 1) {
    if (threadIdx.x < st) red[threadIdx.x] += red[threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}
// out[0..63] partials, out[64] the dot product
void dot_partial(cudaStream_t s, int64_t n, const double *a, const double *b, double *out) {
  dot_part_kernel<<<64, 256, 0, s>>>(n, a, b, out);
  GPGP_CHECK_LAUNCH();
  sum_vec(s, out, 64, out + 64);
}

__global__ void maxabs_part_kernel(int64_t n, const double *__restrict__ a,
                                   const double *__restrict__ b, double *__restrict__ part) {
  __shared__ double red[256];
  double s = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * 256 + threadIdx.x; i < n; i += (int64_t)gridDim.x * 256) {
    double d = fabs(a[i] - b[i]);
    s = (d > s || isnan(d)) ? d : s;
  }
  red[threadIdx.x] = s;
  __syncthreads();
  for (int st = 128; st > 0; st >>= 1) {
    if (threadIdx.x < st) {
      double o = red[threadIdx.x + st];
      if (o > red[threadIdx.x] || isnan(o)) red[threadIdx.x] = o;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}
__global__ void max_vec_kernel(const double *__restrict__ v, int n, double *__restrict__ out) {
  if (threadIdx.x == 0) {
    double m = 0.0;
    for (int i = 0; i < n; ++i)
      if (v[i] > m || isnan(v[i])) m = v[i];
    out[0] = m;
  }
}
// out[0..63] partials, out[64] = max |a - b|
void max_abs_diff(cudaStream_t s, int64_t n, const double *a, const double *b, double *out) {
  maxabs_part_kernel<<<64, 256, 0, s>>>(n, a, b, out);
  GPGP_CHECK_LAUNCH();
  max_vec_kernel<<<1, 32, 0, s>>>(out, 64, out + 64);
  GPGP_CHECK_LAUNCH();
}

// ---------------------------------------------------------------------------
// Gauss-Hermite nodes and weights for the standard normal (R/quadrature.R:1-34):
// nodes are the roots of the probabilists' Hermite polynomial He_q, weights
// q! / (q^2 He_{q-1}(x)^2). Roots are bracketed on a fine grid and polished by
// bisection + Newton (the reference uses polyroot; both are exact to rounding).
// ---------------------------------------------------------------------------
static void he_eval(int q, double x, double *hq, double *hq1) {
  double p0 = 1.0, p1 = x;
  if (q == 0) {
    *hq = 1.0;
    *hq1 = 0.0;
    return;
  }
  for (int k = 2; k <= q; ++k) {
    double p2 = x * p1 - (k - 1) * p0;
    p0 = p1;
    p1 = p2;
  }
  *hq = p1;
  *hq1 = p0;
}

void gauss_hermite(int q, std::vector<double> *xs, std::vector<double> *ws) {
  xs->clear();
  ws->clear();
  if (q < 1) return;
  const double lim = 2.0 * std::sqrt((double)q) + 2.0;
  const int grid = 20000 * q;
  double prev_x = -lim, prev_v, tmp;
  he_eval(q, prev_x, &prev_v, &tmp);
  for (int g = 1; g <= grid && (int)xs->size() < q; ++g) {
    double x = -lim + 2.0 * lim * g / grid;
    double v;
    he_eval(q, x, &v, &tmp);
    if (v == 0.0 || (v > 0) != (prev_v > 0)) {
      double a = prev_x, b = x, fa = prev_v;
      for (int it = 0; it < 200; ++it) {
        double m = 0.5 * (a + b), fm;
        he_eval(q, m, &fm, &tmp);
        if ((fm > 0) == (fa > 0)) {
          a = m;
          fa = fm;
        } else {
          b = m;
        }
      }
      double r = 0.5 * (a + b);
      for (int it = 0; it < 3; ++it) {  // Newton: He_q' = q He_{q-1}
        double h, h1;
        he_eval(q, r, &h, &h1);
        if (h1 != 0.0) r -= h / (q * h1);
      }
      xs->push_back(r);
      prev_x = x + 1e-12;
      he_eval(q, prev_x, &prev_v, &tmp);
      continue;
    }
    prev_x = x;
    prev_v = v;
  }
  double fact = 1.0;
  for (int k = 2; k <= q; ++k) fact *= k;
  for (double r : *xs) {
    double h, h1;
    he_eval(q, r, &h, &h1);
    ws->push_back(fact / ((double)q * q * h1 * h1));
  }
}

}  // namespace gpgp
