// The non-log-concave branch of laplace_iter.method_full (R/laplace.R:40-117)
// and ep_iter.method_full (R/ep.R:50-138), on the device in FP64.
//
// When some pseudo-variance V_i <= 0 (a non-log-concave likelihood such as
// lik_betabinom, or an EP site with negative precision), B = I + V^-1/2 K V^-1/2
// does not exist. The reference then splits the sites into good (V > 0) and bad
// ones: p(y) = p(y_good) p(y_bad | y_good). The good sites get the ordinary B
// factorisation; the bad sites' prior given the good ones is N(pred_mean,
// pred_cov), with Lk = chol(pred_cov) and A = I + Lk^T V_bad^-1 Lk; the final
// alpha = (K + diag(V))^-1 z comes from an LU of K + diag(V) (Matrix::lu).
//
// Here the LU of the whole n x n matrix is replaced by block elimination with
// the good sites' Cholesky factor, which the split computes anyway:
//   K + V = [C1 K12; K21 K22 + V2],  C1 = K11 + V1 = s1^-1 L1 L1^T s1^-1,
//   S = K22 + V2 - K21 C1^-1 K12 = pred_cov + V2 (nbad x nbad, indefinite),
//   a2 = S^-1 (z2 - pred_mean),  a1 = alpha1 - C1^-1 K12 a2,
// so only the small Schur complement S needs an LU with pivoting. The same
// blocks give the predictive variance k^T (K + V)^-1 k = |w1|^2 + u^T S^-1 u with
// w1 = L1^-1 s1 k1 and u = aux^T w1 - k2, aux = L1^-1 s1 K12, and the EP
// marginals V_i (1 - V_i [(K + V)^-1]_ii).
#include <math.h>

#include <algorithm>
#include <cstring>
#include <memory>
#include <vector>

#include "common.cuh"
#include "model.cuh"

namespace gpgp {
namespace {

inline unsigned gridn(int64_t n) { return (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 4096)); }

// out[a + b ldo] = K[ri[a] + ci[b] ldk]
__global__ void gather2_kernel(const double *__restrict__ K, int64_t ldk, const int *__restrict__ ri, int64_t nr,
                               const int *__restrict__ ci, int64_t nc, double *__restrict__ out, int64_t ldo) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nr * nc; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t a = e % nr, b = e / nr;
    out[a + b * ldo] = K[ri[a] + (int64_t)ci[b] * ldk];
  }
}

// rows idx of the n x nf matrix F (ldf) -> out (m x nf, ld m); v: a vector (nf = 1)
__global__ void gather_rows_kernel(const double *__restrict__ F, int64_t ldf, int64_t nf, const int *__restrict__ idx,
                                   int64_t m, double *__restrict__ out) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < m * nf; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t a = e % m, c = e / m;
    out[a + c * m] = F[idx[a] + c * ldf];
  }
}

__global__ void scatter_kernel(const double *__restrict__ v, const int *__restrict__ idx, int64_t m,
                               double *__restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < m) out[idx[i]] = v[i];
}

// A (nr x nc, lda) rows scaled: A_ij *= s_i
__global__ void rowscale_kernel(int64_t nr, int64_t nc, const double *__restrict__ s, double *__restrict__ A,
                                int64_t lda) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nr * nc; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e % nr, j = e / nr;
    A[i + j * lda] *= s[i];
  }
}

// B = I + s_i (K_ij s_j) on the lower triangle (R/laplace.R:27)
__global__ void make_b_kernel(const double *__restrict__ K, int64_t n, const double *__restrict__ s,
                              double *__restrict__ B) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n * n; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e % n, j = e / n;
    if (i < j) continue;
    const double v = s[i] * (K[i + j * n] * s[j]);
    B[i + j * n] = (i == j) ? 1.0 + v : v;
  }
}

// strict upper triangle set to zero
__global__ void zero_upper_kernel(double *__restrict__ A, int64_t n, int64_t lda) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n * n; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e % n, j = e / n;
    if (i < j) A[i + j * lda] = 0.0;
  }
}

// A = I (n x n)
__global__ void identity_kernel(double *__restrict__ A, int64_t n) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n * n; e += (int64_t)gridDim.x * blockDim.x)
    A[e] = (e % n == e / n) ? 1.0 : 0.0;
}

// A_ii += d_i
__global__ void add_diag_kernel(double *__restrict__ A, int64_t n, int64_t lda, const double *__restrict__ d) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) A[i + i * lda] += d[i];
}

__global__ void recip_kernel(int64_t n, const double *__restrict__ v, double *__restrict__ o) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) o[i] = 1.0 / v[i];
}

// out (nc x nr, ldo) = A^T for A (nr x nc, lda)
__global__ void transpose_kernel(int64_t nr, int64_t nc, const double *__restrict__ A, int64_t lda,
                                 double *__restrict__ out, int64_t ldo) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nr * nc; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e % nr, j = e / nr;
    out[j + i * ldo] = A[i + j * lda];
  }
}

__global__ void rsqrt_kernel(int64_t n, const double *__restrict__ v, double *__restrict__ o) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) o[i] = sqrt(1.0 / v[i]);
}

// o = a * b (elementwise), o = a / b, o = a - b
__global__ void ew_kernel(int64_t n, int op, const double *__restrict__ a, const double *__restrict__ b,
                          double *__restrict__ o) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  o[i] = op == 0 ? a[i] * b[i] : (op == 1 ? a[i] / b[i] : a[i] - b[i]);
}

// per-site EP evidence terms of the good sites (R/ep.R:45-46): logC + 0.5 log(vc + V)
// + 0.5 (mc - z)^2 / (vc + V); of the bad sites (R/ep.R:113-115) log((vc + V) / V)
// replaces log(vc + V)
__global__ void ep_terms_kernel(int64_t m, const int *__restrict__ idx, int bad, const double *__restrict__ logC,
                                const double *__restrict__ vc, const double *__restrict__ mc,
                                const double *__restrict__ z, const double *__restrict__ V,
                                double *__restrict__ out) {
  const int64_t a = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= m) return;
  const int64_t i = idx[a];
  const double sv = vc[i] + V[i];
  const double dz = mc[i] - z[i];
  out[a] = logC[i] + 0.5 * (bad ? log(sv / V[i]) : log(sv)) + 0.5 * (dz * dz / sv);
}

__global__ void log_kernel(int64_t n, const double *__restrict__ v, double *__restrict__ o) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) o[i] = log(v[i]);
}

// fvar_i = V_i (1 - V_i d_i) (d = diag((K + V)^-1), so that (K + V)^-1 K = I - (K + V)^-1 V)
__global__ void ep_fvar_nlc_kernel(int64_t n, const double *__restrict__ V, const double *__restrict__ d,
                                   double *__restrict__ fvar) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) fvar[i] = V[i] * (1.0 - V[i] * d[i]);
}

// out_j = sum_i A_ij B_ij over rows (nr) for each column j < nc
__global__ void coldot_kernel(int64_t nr, int64_t nc, const double *__restrict__ A, int64_t lda,
                              const double *__restrict__ B, int64_t ldb, double *__restrict__ out) {
  const int64_t j = (int64_t)blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  const int lane = threadIdx.x & 31;
  if (j >= nc) return;
  double acc = 0.0;
  for (int64_t i = lane; i < nr; i += 32) acc = fma(A[i + j * lda], B[i + j * ldb], acc);
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane == 0) out[j] = acc;
}

// diag of the good-good block of (K + V)^-1: s_i^2 |col_i(W1)|^2 + (G H)_ii with
// H = S^-1 G^T (nbad x ngood): out_i = s_i^2 c_i + sum_j G_ij H_ji
__global__ void good_diag_kernel(int64_t ng, int64_t nb, const double *__restrict__ s, const double *__restrict__ c,
                                 const double *__restrict__ G, const double *__restrict__ H, double *__restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ng) return;
  double acc = 0.0;
  for (int64_t j = 0; j < nb; ++j) acc = fma(G[i + j * ng], H[j + i * nb], acc);
  out[i] = s[i] * s[i] * c[i] + acc;
}

__global__ void diag_kernel(int64_t n, const double *__restrict__ A, int64_t lda, double *__restrict__ o) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) o[i] = A[i + i * lda];
}

__global__ void sub3_kernel(int64_t n, const double *__restrict__ a, const double *__restrict__ b,
                            const double *__restrict__ c, double *__restrict__ o) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) o[i] = a[i] - b[i] - c[i];
}

struct Scal {
  DBuf buf;
  double *p = nullptr;
  void init(cudaStream_t s) {
    buf.alloc(s, 512);
    p = buf.p;
  }
};

// x = F^-1 b through the lower factor (Winv: its diagonal-block inverses): forward or
// transposed; b is kept.
void lsolve(cudaStream_t s, const double *L, int64_t n, const double *W, const double *b, double *x, bool trans,
            const int *status) {
  DBuf t;
  t.alloc(s, std::max<int64_t>(n, 1));
  GPGP_CUDA(cudaMemcpyAsync(t.p, b, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
  if (trans)
    trsv_lower_t(s, L, n, n, W, t.p, x, status);
  else
    trsv_lower(s, L, n, n, W, t.p, x, status);
}

double dot(cudaStream_t s, gpgp_ctx *ctx, int64_t n, const double *a, const double *b, double *scratch) {
  dot_partial(s, n, a, b, scratch);  // result at scratch[64]
  return read_scalar(ctx, scratch + 64);
}

double vsum(cudaStream_t s, gpgp_ctx *ctx, int64_t n, const double *v, double *scratch) {
  sum_vec(s, v, n, scratch + 100);
  return read_scalar(ctx, scratch + 100);
}

}  // namespace

// rows idx of F (ldf x nf) -> out (m x nf, leading dimension m)
void gather_rows(cudaStream_t s, const double *F, int64_t ldf, int64_t nf, const int *idx, int64_t m, double *out) {
  if (m <= 0 || nf <= 0) return;
  gather_rows_kernel<<<gridn(m * nf), 256, 0, s>>>(F, ldf, nf, idx, m, out);
  GPGP_CHECK_LAUNCH();
}

// Good (V > 0) and bad site indices of the model's current V, on the host and device.
void split_sites(gpgp_model *m, std::vector<int> *hg, std::vector<int> *hb, IBuf *good, IBuf *bad) {
  cudaStream_t s = m->ctx->stream;
  const int64_t n = m->n;
  std::vector<double> hV(n);
  GPGP_CUDA(cudaMemcpyAsync(hV.data(), m->V.p, n * sizeof(double), cudaMemcpyDeviceToHost, s));
  GPGP_CUDA(cudaStreamSynchronize(s));
  hg->clear();
  hb->clear();
  for (int64_t i = 0; i < n; ++i) (hV[i] > 0.0 ? hg : hb)->push_back((int)i);
  good->alloc(s, std::max<size_t>(hg->size(), 1));
  bad->alloc(s, std::max<size_t>(hb->size(), 1));
  if (!hg->empty())
    GPGP_CUDA(cudaMemcpyAsync(good->p, hg->data(), hg->size() * sizeof(int), cudaMemcpyHostToDevice, s));
  if (!hb->empty())
    GPGP_CUDA(cudaMemcpyAsync(bad->p, hb->data(), hb->size() * sizeof(int), cudaMemcpyHostToDevice, s));
}

// The bad sites' part of the split (R/laplace.R:73-104, R/ep.R:88-116), given their
// prior N(pm, pc) conditional on the good sites: Lk = t(chol(pc)) (its failure is an
// error, as in R), A = I + Lk^T V_bad^-1 Lk (its failure sets *improper: R's -Inf),
// f2hat, and the bad sites' evidence term lml2 (Laplace also lpu2, the term of
// log_post_unnorm). zb, Vb, yb, tb, ob are the bad sites' pseudo-data,
// observations, trials and offsets (tb, ob may be null); bad their indices.
gpgp_status nlc_bad_terms(gpgp_model *m, int64_t nb, const int *bad, const double *pm, const double *pc,
                          const double *zb, const double *Vb, const double *yb, const double *tb, const double *ob,
                          bool ep, const double *logC, double *lml2, double *lpu2, bool *improper) {
  gpgp_ctx *ctx = m->ctx;
  cudaStream_t s = ctx->stream;
  *improper = false;
  Scal sc;
  sc.init(s);
  IBuf status;
  status.alloc(s, 4);
  GPGP_CUDA(cudaMemsetAsync(status.p, 0, 4 * sizeof(int), s));
  int hs = 0;
  DBuf Lk, Wk, ldk, A, Wa, lda_, v1, v2, v3;
  // Lk = t(chol(pred_cov)): an R error when it fails
  const int64_t nbkb = (nb + NB - 1) / NB;
  Lk.alloc(s, nb * nb);
  Wk.alloc(s, nbkb * NB * NB);
  ldk.alloc(s, nbkb + 1);
  GPGP_CUDA(cudaMemcpyAsync(Lk.p, pc, nb * nb * sizeof(double), cudaMemcpyDeviceToDevice, s));
  potrf(s, Lk.p, nb, nb, Wk.p, ldk.p, status.p + 1);
  zero_upper_kernel<<<gridn(nb * nb), 256, 0, s>>>(Lk.p, nb, nb);
  GPGP_CHECK_LAUNCH();
  GPGP_CUDA(cudaMemcpyAsync(&hs, status.p + 1, sizeof(int), cudaMemcpyDeviceToHost, s));
  GPGP_CUDA(cudaStreamSynchronize(s));
  if (hs)
    return fail(ctx, GPGP_ENOT_PD,
                "chol(pred_cov) of the bad sites failed: the posterior of the whole data is not proper");
  // A = I + Lk^T V_bad^-1 Lk; chol(A) failing -> log_evidence = -Inf
  {
    DBuf T;
    T.alloc(s, nb * nb);
    GPGP_CUDA(cudaMemcpyAsync(T.p, Lk.p, nb * nb * sizeof(double), cudaMemcpyDeviceToDevice, s));
    DBuf iv;
    iv.alloc(s, nb);
    recip_kernel<<<g1(nb), 256, 0, s>>>(nb, Vb, iv.p);  // 1 / V_bad
    GPGP_CHECK_LAUNCH();
    rowscale_kernel<<<gridn(nb * nb), 256, 0, s>>>(nb, nb, iv.p, T.p, nb);
    GPGP_CHECK_LAUNCH();
    A.alloc(s, nb * nb);
    identity_kernel<<<gridn(nb * nb), 256, 0, s>>>(A.p, nb);
    GPGP_CHECK_LAUNCH();
    gemm64(s, true, false, nb, nb, nb, 1.0, Lk.p, nb, T.p, nb, 1.0, A.p, nb);
  }
  Wa.alloc(s, nbkb * NB * NB);
  lda_.alloc(s, nbkb + 1);
  potrf(s, A.p, nb, nb, Wa.p, lda_.p, status.p + 2);
  GPGP_CUDA(cudaMemcpyAsync(&hs, status.p + 2, sizeof(int), cudaMemcpyDeviceToHost, s));
  GPGP_CUDA(cudaStreamSynchronize(s));
  if (hs) {
    *improper = true;
    return GPGP_OK;
  }
  // solve_a(v) = A^-1 v through A_chol; alpha2 = Lk^-T solve_a(Lk^T (z_bad / V_bad))
  v1.alloc(s, nb);
  v2.alloc(s, nb);
  v3.alloc(s, nb);
  auto solve_a = [&](const double *in, double *out) {
    lsolve(s, A.p, nb, Wa.p, in, v3.p, false, status.p);
    lsolve(s, A.p, nb, Wa.p, v3.p, out, true, status.p);
  };
  DBuf alpha2, aux2, f2;
  alpha2.alloc(s, nb);
  aux2.alloc(s, nb);
  f2.alloc(s, nb);
  ew_kernel<<<g1(nb), 256, 0, s>>>(nb, 1, zb, Vb, v1.p);
  GPGP_CHECK_LAUNCH();
  gemv64(s, true, nb, nb, 1.0, Lk.p, nb, v1.p, 0.0, v2.p);  // Lk^T v
  solve_a(v2.p, v1.p);
  lsolve(s, Lk.p, nb, Wk.p, v1.p, alpha2.p, true, status.p);
  // aux = Lk^-T Lk^-1 pred_mean; aux = Lk^-T solve_a(Lk^T aux)
  lsolve(s, Lk.p, nb, Wk.p, pm, v1.p, false, status.p);
  lsolve(s, Lk.p, nb, Wk.p, v1.p, v2.p, true, status.p);
  gemv64(s, true, nb, nb, 1.0, Lk.p, nb, v2.p, 0.0, v1.p);
  solve_a(v1.p, v2.p);
  lsolve(s, Lk.p, nb, Wk.p, v2.p, aux2.p, true, status.p);
  // f2hat = pred_cov (alpha2 + aux)
  vec_axpby(s, nb, 1.0, alpha2.p, 1.0, aux2.p);
  gemv64(s, false, nb, nb, 1.0, pc, nb, aux2.p, 0.0, f2.p);
  sum_vec(s, lda_.p, nbkb, sc.p + 310);
  const double invC2_V2_logdet = 2.0 * read_scalar(ctx, sc.p + 310);
  if (!ep) {
    // df2 = |Lk^-1 (f2hat - pred_mean)|^2 (R/laplace.R:98)
    ew_kernel<<<g1(nb), 256, 0, s>>>(nb, 2, f2.p, pm, v1.p);
    GPGP_CHECK_LAUNCH();
    lsolve(s, Lk.p, nb, Wk.p, v1.p, v2.p, false, status.p);
    const double df2 = dot(s, ctx, nb, v2.p, v2.p, sc.p);
    lik_loglik(s, m->lk, nb, f2.p, yb, tb, ob, sc.p + 410, sc.p);
    const double ll2 = read_scalar(ctx, sc.p + 410);
    *lml2 = ll2 - 0.5 * df2 + 0.5 * invC2_V2_logdet;
    *lpu2 = ll2 - 0.5 * df2;
  } else {
    // df2 = d^T Lk^-T solve_a(Lk^T (d / V_bad)), d = pred_mean - z_bad (R/ep.R:108-111)
    DBuf d;
    d.alloc(s, nb);
    ew_kernel<<<g1(nb), 256, 0, s>>>(nb, 2, pm, zb, d.p);
    ew_kernel<<<g1(nb), 256, 0, s>>>(nb, 1, d.p, Vb, v1.p);
    GPGP_CHECK_LAUNCH();
    gemv64(s, true, nb, nb, 1.0, Lk.p, nb, v1.p, 0.0, v2.p);
    solve_a(v2.p, v1.p);
    lsolve(s, Lk.p, nb, Wk.p, v1.p, v2.p, true, status.p);
    const double df2 = dot(s, ctx, nb, d.p, v2.p, sc.p);
    DBuf terms;
    terms.alloc(s, nb);
    ep_terms_kernel<<<g1(nb), 256, 0, s>>>(nb, bad, 1, logC, m->cav_var.p, m->cav_mean.p, m->z.p, m->V.p,
                                           terms.p);
    GPGP_CHECK_LAUNCH();
    const double st = vsum(s, ctx, nb, terms.p, sc.p);
    *lml2 = -0.5 * df2 + 0.5 * invC2_V2_logdet + st;
  }
  return GPGP_OK;
}

// The split of a method_full Laplace (ep = false) or EP (ep = true) iteration.
// Inputs: the fit's K (n x n, jitter included), m->z, m->V, and for EP the site
// terms logC, m->cav_mean, m->cav_var. Outputs alpha, fnew = K alpha, for EP the
// marginal variances fvar, and the log evidence. *improper is set (and nothing
// else written) when chol(A) fails, where the reference returns -Inf. Leaves the
// blocks the prediction needs in m->nlc.
gpgp_status nlc_fit_full(gpgp_model *m, const double *K, const double *logC, bool ep, double *alpha, double *fnew,
                         double *fvar, double *lml, bool *improper) {
  gpgp_ctx *ctx = m->ctx;
  cudaStream_t s = ctx->stream;
  const int64_t n = m->n;
  *improper = false;
  std::vector<double> hV(n);
  GPGP_CUDA(cudaMemcpyAsync(hV.data(), m->V.p, n * sizeof(double), cudaMemcpyDeviceToHost, s));
  GPGP_CUDA(cudaStreamSynchronize(s));
  std::vector<int> hg, hb;
  for (int64_t i = 0; i < n; ++i) (hV[i] > 0.0 ? hg : hb).push_back((int)i);
  const int64_t ng = (int64_t)hg.size(), nb = (int64_t)hb.size();
  if (ng == 0) return fail(ctx, GPGP_EUNSUPPORTED, "every pseudo-variance is <= 0: no good sites to condition on");
  auto st_ = std::unique_ptr<NlcState>(new NlcState());
  NlcState &S = *st_;
  S.ng = ng;
  S.nb = nb;
  S.good.alloc(s, ng);
  S.bad.alloc(s, nb);
  GPGP_CUDA(cudaMemcpyAsync(S.good.p, hg.data(), ng * sizeof(int), cudaMemcpyHostToDevice, s));
  GPGP_CUDA(cudaMemcpyAsync(S.bad.p, hb.data(), nb * sizeof(int), cudaMemcpyHostToDevice, s));
  const double *trials = m->has_trials ? m->trials.p : nullptr;
  const double *offset = m->has_offset ? m->offset.p : nullptr;
  Scal sc;
  sc.init(s);
  IBuf status;
  status.alloc(s, 4);
  GPGP_CUDA(cudaMemsetAsync(status.p, 0, 4 * sizeof(int), s));
  // ---- the good sites: ordinary B factorisation (the recursive laplace_iter / ep_iter)
  DBuf Kg, zg, Vg, yg, tg, og, a1, f1, tmp;
  Kg.alloc(s, ng * ng);
  gather2_kernel<<<gridn(ng * ng), 256, 0, s>>>(K, n, S.good.p, ng, S.good.p, ng, Kg.p, ng);
  GPGP_CHECK_LAUNCH();
  auto gatv = [&](DBuf &dst, const double *src, const int *idx, int64_t cnt) {
    dst.alloc(s, std::max<int64_t>(cnt, 1));
    if (cnt) {
      gather_rows_kernel<<<gridn(cnt), 256, 0, s>>>(src, n, 1, idx, cnt, dst.p);
      GPGP_CHECK_LAUNCH();
    }
  };
  gatv(zg, m->z.p, S.good.p, ng);
  gatv(Vg, m->V.p, S.good.p, ng);
  gatv(yg, m->y.p, S.good.p, ng);
  if (trials) gatv(tg, trials, S.good.p, ng);
  if (offset) gatv(og, offset, S.good.p, ng);
  S.sg.alloc(s, ng);
  rsqrt_kernel<<<g1(ng), 256, 0, s>>>(ng, Vg.p, S.sg.p);
  GPGP_CHECK_LAUNCH();
  const int64_t nbk1 = (ng + NB - 1) / NB;
  S.L1.alloc(s, ng * ng);
  S.W1.alloc(s, nbk1 * NB * NB);
  DBuf ld1;
  ld1.alloc(s, nbk1 + 1);
  make_b_kernel<<<gridn(ng * ng), 256, 0, s>>>(Kg.p, ng, S.sg.p, S.L1.p);
  GPGP_CHECK_LAUNCH();
  potrf(s, S.L1.p, ng, ng, S.W1.p, ld1.p, status.p);
  int hs = 0;
  GPGP_CUDA(cudaMemcpyAsync(&hs, status.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  GPGP_CUDA(cudaStreamSynchronize(s));
  if (hs) return fail(ctx, GPGP_ENOT_PD, "Cholesky factorisation of the good sites: not positive definite");
  // alpha1 = s L^-T L^-1 (s z)
  a1.alloc(s, ng);
  f1.alloc(s, ng);
  tmp.alloc(s, std::max(ng, nb) + 1);
  ew_kernel<<<g1(ng), 256, 0, s>>>(ng, 0, S.sg.p, zg.p, tmp.p);
  GPGP_CHECK_LAUNCH();
  lsolve(s, S.L1.p, ng, S.W1.p, tmp.p, f1.p, false, status.p);
  lsolve(s, S.L1.p, ng, S.W1.p, f1.p, tmp.p, true, status.p);
  ew_kernel<<<g1(ng), 256, 0, s>>>(ng, 0, S.sg.p, tmp.p, a1.p);
  GPGP_CHECK_LAUNCH();
  gemv64(s, false, ng, ng, 1.0, Kg.p, ng, a1.p, 0.0, f1.p);
  sum_vec(s, ld1.p, nbk1, sc.p + 300);
  const double logdetL1 = read_scalar(ctx, sc.p + 300);
  double lml1;
  if (!ep) {
    // R/laplace.R:33-38 on the good sites: loglik - 0.5 f^T alpha - 0.5 (2 sum log L_ii)
    lik_loglik(s, m->lk, ng, f1.p, yg.p, trials ? tg.p : nullptr, offset ? og.p : nullptr, sc.p + 400, sc.p);
    const double ll = read_scalar(ctx, sc.p + 400);
    const double fa = dot(s, ctx, ng, f1.p, a1.p, sc.p);
    lml1 = ll - 0.5 * fa - 0.5 * (2.0 * logdetL1);
  } else {
    // R/ep.R:43-49 on the good sites
    DBuf terms;
    terms.alloc(s, ng);
    ep_terms_kernel<<<g1(ng), 256, 0, s>>>(ng, S.good.p, 0, logC, m->cav_var.p, m->cav_mean.p, m->z.p, m->V.p,
                                           terms.p);
    GPGP_CHECK_LAUNCH();
    const double st = vsum(s, ctx, ng, terms.p, sc.p);
    log_kernel<<<g1(ng), 256, 0, s>>>(ng, Vg.p, terms.p);
    GPGP_CHECK_LAUNCH();
    const double slv = vsum(s, ctx, ng, terms.p, sc.p);
    const double za = dot(s, ctx, ng, zg.p, a1.p, sc.p);
    lml1 = -0.5 * (2.0 * logdetL1 + slv) - 0.5 * za + st;
  }
  // ---- the bad sites' prior given the good ones
  DBuf K12, K22, pm, pc, zb, Vb, yb, tb, ob;
  K12.alloc(s, ng * nb);
  K22.alloc(s, nb * nb);
  gather2_kernel<<<gridn(ng * nb), 256, 0, s>>>(K, n, S.good.p, ng, S.bad.p, nb, K12.p, ng);
  GPGP_CHECK_LAUNCH();
  gather2_kernel<<<gridn(nb * nb), 256, 0, s>>>(K, n, S.bad.p, nb, S.bad.p, nb, K22.p, nb);
  GPGP_CHECK_LAUNCH();
  gatv(zb, m->z.p, S.bad.p, nb);
  gatv(Vb, m->V.p, S.bad.p, nb);
  gatv(yb, m->y.p, S.bad.p, nb);
  if (trials) gatv(tb, trials, S.bad.p, nb);
  if (offset) gatv(ob, offset, S.bad.p, nb);
  pm.alloc(s, nb);
  gemv64(s, true, ng, nb, 1.0, K12.p, ng, a1.p, 0.0, pm.p);  // pred_mean = K21 alpha1
  // aux = L1^-1 s1 K12 (= forwardsolve(C_chol, t(K21)))
  S.aux.alloc(s, ng * nb);
  GPGP_CUDA(cudaMemcpyAsync(S.aux.p, K12.p, ng * nb * sizeof(double), cudaMemcpyDeviceToDevice, s));
  rowscale_kernel<<<gridn(ng * nb), 256, 0, s>>>(ng, nb, S.sg.p, S.aux.p, ng);
  GPGP_CHECK_LAUNCH();
  {
    DBuf t;
    t.alloc(s, (size_t)NB * nb);
    trsm_lower(s, S.L1.p, ng, ng, S.W1.p, S.aux.p, nb, ng, t.p, status.p);
  }
  // pred_cov = K22 - aux^T aux
  pc.alloc(s, nb * nb);
  GPGP_CUDA(cudaMemcpyAsync(pc.p, K22.p, nb * nb * sizeof(double), cudaMemcpyDeviceToDevice, s));
  gemm64(s, true, false, nb, nb, ng, -1.0, S.aux.p, ng, S.aux.p, ng, 1.0, pc.p, nb);
  double lml2 = 0.0, lpu2 = 0.0;
  {
    gpgp_status s2 = nlc_bad_terms(m, nb, S.bad.p, pm.p, pc.p, zb.p, Vb.p, yb.p, trials ? tb.p : nullptr,
                                   offset ? ob.p : nullptr, ep, logC, &lml2, &lpu2, improper);
    if (s2 != GPGP_OK) return s2;
    if (*improper) {
      *lml = -INFINITY;
      return GPGP_OK;
    }
  }
  DBuf v1;
  v1.alloc(s, nb);
  // ---- the whole data: S = pred_cov + diag(V_bad), LU; a2 = S^-1 (z_bad - pred_mean),
  // a1 = alpha1 - s1 L1^-T (aux a2)
  S.Slu.alloc(s, nb * nb);
  S.piv.alloc(s, nb);
  GPGP_CUDA(cudaMemcpyAsync(S.Slu.p, pc.p, nb * nb * sizeof(double), cudaMemcpyDeviceToDevice, s));
  add_diag_kernel<<<g1(nb), 256, 0, s>>>(S.Slu.p, nb, nb, Vb.p);
  GPGP_CHECK_LAUNCH();
  getrf(s, S.Slu.p, nb, nb, S.piv.p, status.p + 3);
  ew_kernel<<<g1(nb), 256, 0, s>>>(nb, 2, zb.p, pm.p, v1.p);
  GPGP_CHECK_LAUNCH();
  getrs(s, S.Slu.p, nb, nb, S.piv.p, v1.p, 1, nb, status.p + 3);
  GPGP_CUDA(cudaMemcpyAsync(&hs, status.p + 3, sizeof(int), cudaMemcpyDeviceToHost, s));
  GPGP_CUDA(cudaStreamSynchronize(s));
  if (hs) return fail(ctx, GPGP_ENOT_PD, "K + diag(V) is singular (LU of the bad sites' Schur complement)");
  DBuf w;
  w.alloc(s, ng);
  gemv64(s, false, ng, nb, 1.0, S.aux.p, ng, v1.p, 0.0, w.p);  // aux a2
  lsolve(s, S.L1.p, ng, S.W1.p, w.p, tmp.p, true, status.p);
  ew_kernel<<<g1(ng), 256, 0, s>>>(ng, 0, S.sg.p, tmp.p, w.p);
  ew_kernel<<<g1(ng), 256, 0, s>>>(ng, 2, a1.p, w.p, w.p);  // a1
  GPGP_CHECK_LAUNCH();
  scatter_kernel<<<g1(ng), 256, 0, s>>>(w.p, S.good.p, ng, alpha);
  scatter_kernel<<<g1(nb), 256, 0, s>>>(v1.p, S.bad.p, nb, alpha);
  GPGP_CHECK_LAUNCH();
  gemv64(s, false, n, n, 1.0, K, n, alpha, 0.0, fnew);
  if (ep) {
    // diag((K + V)^-1): good sites s_i^2 |col_i(W1)|^2 + (G S^-1 G^T)_ii with
    // G = C1^-1 K12 = s1 W1^T aux (W1 = L1^-1); bad sites diag(S^-1)
    DBuf W1full, tt, csq, G, H, dgood, Sinv, dbad, d;
    W1full.alloc(s, ng * ng);
    tt.alloc(s, (size_t)NB * ng);
    trtri_lower(s, S.L1.p, ng, ng, S.W1.p, W1full.p, ng, tt.p, status.p);
    csq.alloc(s, ng);
    col_sumsq_lower(s, W1full.p, ng, ng, csq.p);
    G.alloc(s, ng * nb);
    gemm64(s, true, false, ng, nb, ng, 1.0, W1full.p, ng, S.aux.p, ng, 0.0, G.p, ng);
    rowscale_kernel<<<gridn(ng * nb), 256, 0, s>>>(ng, nb, S.sg.p, G.p, ng);
    GPGP_CHECK_LAUNCH();
    H.alloc(s, nb * ng);
    transpose_kernel<<<gridn(ng * nb), 256, 0, s>>>(ng, nb, G.p, ng, H.p, nb);  // H = G^T
    GPGP_CHECK_LAUNCH();
    getrs(s, S.Slu.p, nb, nb, S.piv.p, H.p, ng, nb, status.p + 3);  // H = S^-1 G^T
    dgood.alloc(s, ng);
    good_diag_kernel<<<g1(ng), 256, 0, s>>>(ng, nb, S.sg.p, csq.p, G.p, H.p, dgood.p);
    GPGP_CHECK_LAUNCH();
    Sinv.alloc(s, nb * nb);
    identity_kernel<<<gridn(nb * nb), 256, 0, s>>>(Sinv.p, nb);
    GPGP_CHECK_LAUNCH();
    getrs(s, S.Slu.p, nb, nb, S.piv.p, Sinv.p, nb, nb, status.p + 3);
    dbad.alloc(s, nb);
    diag_kernel<<<g1(nb), 256, 0, s>>>(nb, Sinv.p, nb, dbad.p);
    GPGP_CHECK_LAUNCH();
    d.alloc(s, n);
    scatter_kernel<<<g1(ng), 256, 0, s>>>(dgood.p, S.good.p, ng, d.p);
    scatter_kernel<<<g1(nb), 256, 0, s>>>(dbad.p, S.bad.p, nb, d.p);
    GPGP_CHECK_LAUNCH();
    ep_fvar_nlc_kernel<<<g1(n), 256, 0, s>>>(n, m->V.p, d.p, fvar);
    GPGP_CHECK_LAUNCH();
  }
  *lml = lml1 + lml2;
  m->nlc = std::move(st_);
  return GPGP_OK;
}

// var = diag(Ktt) - diag(Kt (K + V)^-1 Kt^T) (R/gp_pred.R:220-223) through the blocks:
// k^T (K + V)^-1 k = |w1|^2 + u^T S^-1 u, w1 = L1^-1 s1 k1, u = aux^T w1 - k2.
void nlc_pred_var(gpgp_model *m, const double *Ft, int64_t mt, uint32_t gm, double *var) {
  NlcState &S = *m->nlc;
  cudaStream_t s = m->ctx->stream;
  const int64_t ng = S.ng, nb = S.nb, nf = std::max(1, m->dk.nfeat);
  if (!S.Fg.p) {
    S.Fg.alloc(s, ng * nf);
    gather_rows_kernel<<<gridn(ng * nf), 256, 0, s>>>(m->F.p, m->n, nf, S.good.p, ng, S.Fg.p);
    GPGP_CHECK_LAUNCH();
    S.Fb.alloc(s, std::max<int64_t>(nb, 1) * nf);
    if (nb) {
      gather_rows_kernel<<<gridn(nb * nf), 256, 0, s>>>(m->F.p, m->n, nf, S.bad.p, nb, S.Fb.p);
      GPGP_CHECK_LAUNCH();
    }
  }
  const int64_t chunk = std::max<int64_t>(1, std::min<int64_t>(mt, (int64_t)(1ll << 27) / std::max<int64_t>(ng, 1)));
  DBuf R, U, X, tmp, t1, t2, kd;
  R.alloc(s, ng * chunk);
  U.alloc(s, std::max<int64_t>(nb, 1) * chunk);
  X.alloc(s, std::max<int64_t>(nb, 1) * chunk);
  tmp.alloc(s, (size_t)NB * chunk);
  t1.alloc(s, mt);
  t2.alloc(s, mt);
  kd.alloc(s, mt);
  IBuf status;
  status.alloc(s, 1);
  GPGP_CUDA(cudaMemsetAsync(status.p, 0, sizeof(int), s));
  GPGP_CUDA(cudaMemsetAsync(t2.p, 0, mt * sizeof(double), s));
  for (int64_t c0 = 0; c0 < mt; c0 += chunk) {
    const int64_t mc = std::min(chunk, mt - c0);
    cov_matrix(s, m->dk, gm, S.Fg.p, ng, ng, Ft + c0, mt, mc, R.p, ng, COV_ROWSCALE, 0, 0, 0.0, S.sg.p);
    trsm_lower(s, S.L1.p, ng, ng, S.W1.p, R.p, mc, ng, tmp.p, status.p);
    col_sumsq(s, R.p, ng, mc, ng, t1.p + c0);
    if (nb) {
      cov_matrix(s, m->dk, gm, S.Fb.p, nb, nb, Ft + c0, mt, mc, U.p, nb, COV_FULL, 0, 0, 0.0, nullptr);
      gemm64(s, true, false, nb, mc, ng, 1.0, S.aux.p, ng, R.p, ng, -1.0, U.p, nb);
      GPGP_CUDA(cudaMemcpyAsync(X.p, U.p, nb * mc * sizeof(double), cudaMemcpyDeviceToDevice, s));
      getrs(s, S.Slu.p, nb, nb, S.piv.p, X.p, mc, nb, status.p);
      coldot_kernel<<<(unsigned)((mc + 7) / 8), 256, 0, s>>>(nb, mc, U.p, nb, X.p, nb, t2.p + c0);
      GPGP_CHECK_LAUNCH();
    }
  }
  cov_diag(s, m->dk, gm, Ft, mt, Ft, mt, mt, kd.p);
  sub3_kernel<<<g1(mt), 256, 0, s>>>(mt, kd.p, t1.p, t2.p, var);
  GPGP_CHECK_LAUNCH();
}

}  // namespace gpgp
