// FITC (method_fitc) on the device: set-up of the inducing-point algebra,
// Laplace and EP iterations through the inversion lemma, prediction and the
// training-point posterior variances used by LOO.
//
// Restates fit_laplace.method_fitc / fit_ep.method_fitc (R/gp_fit.R:101-123,
// 163-188), laplace_iter.method_fitc / laplace.method_fitc
// (R/laplace.R:122-152, 299-325), ep_iter.method_fitc / ep.method_fitc
// (R/ep.R:148-185, 274-279, 333-374), inv_lemma_get / inv_lemma_solve
// (R/linear_algebra.R:3-126) and gp_pred_post.method_fitc
// (R/gp_pred.R:234-296). Every product is O(n M^2) or less; n x n matrices
// never appear. Solves with the M x M factors of K_z and of the lemma's
// C_m = K_z + U^T S^-1 U are substitutions, as forwardsolve/backsolve do,
// applied to the rows of n x M matrices (one thread per row, coalesced):
// X = K(x, z) L_z^-T is the transpose of the reference's
// forwardsolve(Kz_chol, t(Kxz)). Explicit inverses of these often
// ill-conditioned factors would cost accuracy. The n x M Gram product
// U^T S^-1 U uses the sliced tensor-core GEMM in mixed precision.
#include <math.h>

#include <algorithm>
#include <vector>

#include "common.cuh"
#include "model.cuh"

namespace gpgp {
namespace {

// out[i, m] = X[i, m] / v[i]  (n x M, column-major)
__global__ void div_rows_kernel(int64_t n, int64_t M, const double *__restrict__ X,
                                const double *__restrict__ v, double *__restrict__ out) {
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n * M;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = idx % n;
    out[idx] = X[idx] / v[i];
  }
}

// out[m, i] = X[i, m] * v[i]  (X n x M -> out M x n)
__global__ void transpose_scale_kernel(int64_t n, int64_t M, const double *__restrict__ X,
                                       const double *__restrict__ v, double *__restrict__ out) {
  __shared__ double t[32][33];
  const int64_t i0 = (int64_t)blockIdx.x * 32, m0 = (int64_t)blockIdx.y * 32;
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    const int64_t i = i0 + threadIdx.x, m = m0 + r;
    t[r][threadIdx.x] = (i < n && m < M) ? X[i + m * n] * v[i] : 0.0;
  }
  __syncthreads();
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    const int64_t m = m0 + threadIdx.x, i = i0 + r;
    if (i < n && m < M) out[m + i * M] = t[threadIdx.x][r];
  }
}

// C = K + 0.5 (V + V^T)  (M x M)
__global__ void sym_add_kernel(int64_t M, const double *__restrict__ K, const double *__restrict__ V,
                               double *__restrict__ C) {
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < M * M;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = idx % M, j = idx / M;
    C[idx] = K[idx] + 0.5 * (V[idx] + V[j + i * M]);
  }
}

// y[i] = a[i] + b[i] * c[i]
__global__ void fma_vec_kernel(int64_t n, const double *__restrict__ a, const double *__restrict__ b,
                               const double *__restrict__ c, double *__restrict__ y) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = a[i] + b[i] * c[i];
}

// y[i] = a[i] / b[i]
__global__ void div_vec_kernel(int64_t n, const double *__restrict__ a, const double *__restrict__ b,
                               double *__restrict__ y) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = a[i] / b[i];
}

// out[i] = a[i] + s * b[i]
__global__ void axpy_vec_kernel(int64_t n, const double *__restrict__ a, double s,
                                const double *__restrict__ b, double *__restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = a[i] + s * b[i];
}

// out[i] = sum_m A[m, i] * B[m, i]  (A, B are M x n; one warp per column)
__global__ void coldot_kernel(int64_t M, int64_t n, const double *__restrict__ A,
                              const double *__restrict__ B, double *__restrict__ out) {
  const int lane = threadIdx.x & 31;
  const int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (i >= n) return;
  double s = 0.0;
  for (int64_t m = lane; m < M; m += 32) s = fma(A[m + i * M], B[m + i * M], s);
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if (lane == 0) out[i] = s;
}

// out[i] = sum_m X[i, m] * Y[m, i]  (X n x M, Y M x n)
__global__ void rowdot_kernel(int64_t M, int64_t n, const double *__restrict__ X,
                              const double *__restrict__ Y, double *__restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = 0.0;
  for (int64_t m = 0; m < M; ++m) s = fma(X[i + m * n], Y[m + i * M], s);
  out[i] = s;
}

// out[i] = sum_m X[i, m] * Y[i, m]  (X, Y are n x M)
__global__ void rowdot_nn_kernel(int64_t M, int64_t n, const double *__restrict__ X,
                                 const double *__restrict__ Y, double *__restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = 0.0;
  for (int64_t m = 0; m < M; ++m) s = fma(X[i + m * n], Y[i + m * n], s);
  out[i] = s;
}

// out[i, m] = X[i, m] * v[i]  (n x M)
__global__ void scale_rows_kernel(int64_t n, int64_t M, const double *__restrict__ X,
                                  const double *__restrict__ v, double *__restrict__ out) {
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n * M;
       idx += (int64_t)gridDim.x * blockDim.x)
    out[idx] = X[idx] * v[idx % n];
}

// A[m, i] *= v[i]  (A is M x n)
__global__ void scale_cols_kernel(int64_t M, int64_t n, double *__restrict__ A,
                                  const double *__restrict__ v) {
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < M * n;
       idx += (int64_t)gridDim.x * blockDim.x)
    A[idx] *= v[idx / M];
}

// D_i = (Kdiag_i + jitter) - cs_i  (cs may be null)
__global__ void fitc_d_kernel(int64_t n, const double *__restrict__ Kdiag, double jit,
                              const double *__restrict__ cs, double *__restrict__ D) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) D[i] = cs ? (Kdiag[i] + jit) - cs[i] : Kdiag[i] + jit;
}

// A_ii += d_i (n x n, leading dimension n)
__global__ void add_diag2_kernel(double *__restrict__ A, int64_t n, const double *__restrict__ d) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) A[i + i * n] += d[i];
}

__global__ void fill_kernel(int64_t n, double v, double *__restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = v;
}

__global__ void loo_moments_kernel(int64_t n, const double *__restrict__ pv,
                                   const double *__restrict__ V, const double *__restrict__ z,
                                   const double *__restrict__ fh, double *__restrict__ lm,
                                   double *__restrict__ lv) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    const double grad = (z[i] - fh[i]) / V[i];
    const double v = 1.0 / (1.0 / pv[i] - 1.0 / V[i]);
    lv[i] = v;
    lm[i] = fh[i] - v * grad;
  }
}

__global__ void check_positive2_kernel(int64_t n, const double *__restrict__ V, int *flag) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    if (isnan(V[i])) atomicOr(flag, 2);
    else if (!(V[i] > 0.0)) atomicOr(flag, 4);
  }
}

__global__ void log_vec2_kernel(int64_t n, const double *__restrict__ v, double *__restrict__ o) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) o[i] = log(v[i]);
}

__global__ void recip2_kernel(int64_t n, const double *__restrict__ v, double *__restrict__ o) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) o[i] = 1.0 / v[i];
}

__global__ void ep_terms2_kernel(int64_t n, const double *__restrict__ logC,
                                 const double *__restrict__ vc, const double *__restrict__ mc,
                                 const double *__restrict__ z, const double *__restrict__ V,
                                 double *__restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    const double sv = vc[i] + V[i];
    const double dz = mc[i] - z[i];
    out[i] = logC[i] + 0.5 * log(sv) + 0.5 * (dz * dz / sv);
  }
}

unsigned gs(int64_t n) { return (unsigned)std::min<int64_t>(std::max<int64_t>(1, (n + 255) / 256), 8192); }

// Scalar reductions on a small device scratch
struct Red {
  DBuf b;
  gpgp_ctx *ctx;
  explicit Red(gpgp_ctx *c) : ctx(c) { b.alloc(c->stream, 512); }
  double sum(const double *v, int64_t n, int slot) {
    sum_vec(ctx->stream, v, n, b.p + 300 + slot);
    return read_scalar(ctx, b.p + 300 + slot);
  }
  double dot(const double *a, const double *c, int64_t n) {
    dot_partial(ctx->stream, n, a, c, b.p);
    return read_scalar(ctx, b.p + 64);
  }
};

// M x M Cholesky (blocked, substitution panels); returns the failing pivot
// (0 = ok) and sum log L_ii
int64_t chol_small(gpgp_ctx *ctx, double *A, int64_t M, double *Wblk, double *logdet_out) {
  cudaStream_t st = ctx->stream;
  DBuf part;
  part.alloc(st, (M + NB - 1) / NB + 1);
  IBuf status;
  status.alloc(st, 1);
  GPGP_CUDA(cudaMemsetAsync(status.p, 0, sizeof(int), st));
  potrf(st, A, M, M, Wblk, part.p, status.p);
  DBuf out;
  out.alloc(st, 1);
  sum_vec(st, part.p, (M + NB - 1) / NB, out.p);
  int h = 0;
  GPGP_CUDA(cudaMemcpyAsync(&h, status.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  *logdet_out = read_scalar(ctx, out.p);
  return h;
}

// rows of B (n x M) times C_m^-1 = L_m^-T L_m^-1: two substitution passes
void rows_times_cminv(gpgp_model *m, const double *B, double *X, int64_t n) {
  FitcState &f = *m->fitc;
  cudaStream_t st = m->ctx->stream;
  tri_rows(st, f.Lm.p, f.M, f.M, B, n, X, n, n, 0);
  tri_rows(st, f.Lm.p, f.M, f.M, X, n, X, n, n, 1);
}

// U^T B for U = Kxz, B both n x M, on the FP64 pipe in both precisions: the
// lemma's C_m inherits K_z's conditioning (~1e4 and more), so BF16-sliced
// products move its log-determinant by ~1e-5 relative at n = 65536, and the
// Gram (2 n M^2 flops, split over K) is a small part of a FITC fit anyway.
void gram_tn(gpgp_model *m, const double *A, const double *B, int64_t n, int64_t M, double *C) {
  gemm64(m->ctx->stream, true, false, M, M, n, 1.0, A, n, B, n, 0.0, C, M);
}

// The lemma for the current S (R/linear_algebra.R:3-43): iDU = Kxz / S, C_m and its
// factor, logdet = sum log S - 2 sum log diag(Lz) + 2 sum log diag(Lm).
// Returns false when C_m is not positive definite.
bool lemma_get(gpgp_model *m, Red &red, double logdet_z) {
  FitcState &f = *m->fitc;
  cudaStream_t st = m->ctx->stream;
  const int64_t n = m->n, M = f.M;
  div_rows_kernel<<<gs(n * M), 256, 0, st>>>(n, M, f.Kxz.p, f.S.p, f.iDU.p);
  GPGP_CHECK_LAUNCH();
  DBuf VDU;
  VDU.alloc(st, (size_t)M * M);
  gram_tn(m, f.Kxz.p, f.iDU.p, n, M, VDU.p);
  sym_add_kernel<<<gs(M * M), 256, 0, st>>>(M, f.Kz.p, VDU.p, f.Cm.p);
  GPGP_CHECK_LAUNCH();
  GPGP_CUDA(cudaMemcpyAsync(f.Lm.p, f.Cm.p, M * M * sizeof(double), cudaMemcpyDeviceToDevice, st));
  double ldm = 0.0;
  if (chol_small(m->ctx, f.Lm.p, M, f.Wm_blk.p, &ldm) != 0) return false;
  DBuf lS;
  lS.alloc(st, n);
  log_vec2_kernel<<<g1(n), 256, 0, st>>>(n, f.S.p, lS.p);
  GPGP_CHECK_LAUNCH();
  const double slogS = red.sum(lS.p, n, 1);
  f.logdet = slogS - 2.0 * logdet_z + 2.0 * ldm;
  f.have_pred_cache = false;
  return true;
}

// inv_lemma_solve(C_inv, rhs) for a vector (R/linear_algebra.R:112-122):
// out = rhs / S - iDU C_m^-1 (iDU^T rhs)
void lemma_solve_vec(gpgp_model *m, const double *rhs, double *out) {
  FitcState &f = *m->fitc;
  cudaStream_t st = m->ctx->stream;
  const int64_t n = m->n, M = f.M;
  DBuf t, q;
  t.alloc(st, M);
  q.alloc(st, n);
  gemv64(st, true, n, M, 1.0, f.iDU.p, n, rhs, 0.0, t.p);  // iDU^T rhs
  tri_vec(st, f.Lm.p, M, M, t.p, t.p, false);              // C_m^-1 t by two substitutions
  tri_vec(st, f.Lm.p, M, M, t.p, t.p, true);
  gemv64(st, false, n, M, 1.0, f.iDU.p, n, t.p, 0.0, q.p);  // iDU u
  div_vec_kernel<<<g1(n), 256, 0, st>>>(n, rhs, f.S.p, out);
  GPGP_CHECK_LAUNCH();
  vec_axpby(st, n, -1.0, q.p, 1.0, out);
}

// fhat = Kxz Kz^-1 (Kxz^T alpha) + D alpha (R/laplace.R:133)
void fitc_fmean(gpgp_model *m, const double *alpha, double *fhat) {
  FitcState &f = *m->fitc;
  cudaStream_t st = m->ctx->stream;
  const int64_t n = m->n, M = f.M;
  DBuf w, q;
  w.alloc(st, M);
  q.alloc(st, n);
  gemv64(st, true, n, M, 1.0, f.Kxz.p, n, alpha, 0.0, w.p);  // Kxz^T alpha
  tri_vec(st, f.Lz.p, M, M, w.p, w.p, false);               // forwardsolve(Kz_chol, .)
  tri_vec(st, f.Lz.p, M, M, w.p, w.p, true);                // backsolve(t(Kz_chol), .)
  gemv64(st, false, n, M, 1.0, f.Kxz.p, n, w.p, 0.0, q.p);  // Kxz w
  fma_vec_kernel<<<g1(n), 256, 0, st>>>(n, q.p, f.D.p, alpha, fhat);
  GPGP_CHECK_LAUNCH();
}

// The evidence of a non-log-concave FITC iteration (R/laplace.R:151-216,
// R/ep.R:186-255): the good sites' lemma fit (the recursive laplace_iter / ep_iter),
// the bad sites' prior given them through the inducing inputs,
//   K21 = X_bad X_good^T, prior_cov = X_bad X_bad^T + diag(D_bad),
//   pred_cov = prior_cov - K21 inv_lemma_solve(C_inv_good, K21^T),
// and the shared bad-site terms (nlc.cu). *failed: a Cholesky inside the reference's
// tryCatch failed (the fit's evidence is -Inf); *improper: chol(A) failed.
gpgp_status fitc_nlc_terms(gpgp_model *m, Red &red, double logdet_z, bool ep, const double *logC, double *lml,
                           double *lpu, bool *improper, bool *failed) {
  FitcState &f = *m->fitc;
  gpgp_ctx *ctx = m->ctx;
  cudaStream_t st = ctx->stream;
  const int64_t n = m->n, M = f.M;
  *improper = *failed = false;
  std::vector<int> hg, hb;
  IBuf good, bad;
  split_sites(m, &hg, &hb, &good, &bad);
  const int64_t ng = (int64_t)hg.size(), nb = (int64_t)hb.size();
  if (ng == 0) return fail(ctx, GPGP_EUNSUPPORTED, "every pseudo-variance is <= 0: no good sites to condition on");
  const double *trials = m->has_trials ? m->trials.p : nullptr;
  const double *offset = m->has_offset ? m->offset.p : nullptr;
  auto gat = [&](DBuf &dst, const double *src, int64_t ld, int64_t nf, const IBuf &idx, int64_t cnt) {
    dst.alloc(st, std::max<int64_t>(cnt, 1) * nf);
    gather_rows(st, src, ld, nf, idx.p, cnt, dst.p);
  };
  DBuf Ug, Xg, Xb, Dg, Vg, zg, yg, tg, og, Db, Vb, zb, yb, tb, ob;
  gat(Ug, f.Kxz.p, n, M, good, ng);
  gat(Xg, f.X.p, n, M, good, ng);
  gat(Xb, f.X.p, n, M, bad, nb);
  gat(Dg, f.D.p, n, 1, good, ng);
  gat(Vg, m->V.p, n, 1, good, ng);
  gat(zg, m->z.p, n, 1, good, ng);
  gat(yg, m->y.p, n, 1, good, ng);
  gat(Db, f.D.p, n, 1, bad, nb);
  gat(Vb, m->V.p, n, 1, bad, nb);
  gat(zb, m->z.p, n, 1, bad, nb);
  gat(yb, m->y.p, n, 1, bad, nb);
  if (trials) {
    gat(tg, trials, n, 1, good, ng);
    gat(tb, trials, n, 1, bad, nb);
  }
  if (offset) {
    gat(og, offset, n, 1, good, ng);
    gat(ob, offset, n, 1, bad, nb);
  }
  // the good sites' lemma: S = D + V, iDU = U / S, C_m = K_z + U^T S^-1 U
  DBuf Sg, iDUg, VDU, Cm, Lm, Wm, a1, t, q, fg, lS;
  Sg.alloc(st, ng);
  axpy_vec_kernel<<<g1(ng), 256, 0, st>>>(ng, Dg.p, 1.0, Vg.p, Sg.p);
  GPGP_CHECK_LAUNCH();
  iDUg.alloc(st, ng * M);
  div_rows_kernel<<<gs(ng * M), 256, 0, st>>>(ng, M, Ug.p, Sg.p, iDUg.p);
  GPGP_CHECK_LAUNCH();
  VDU.alloc(st, M * M);
  gemm64(st, true, false, M, M, ng, 1.0, Ug.p, ng, iDUg.p, ng, 0.0, VDU.p, M);
  Cm.alloc(st, M * M);
  sym_add_kernel<<<gs(M * M), 256, 0, st>>>(M, f.Kz.p, VDU.p, Cm.p);
  GPGP_CHECK_LAUNCH();
  Lm.alloc(st, M * M);
  Wm.alloc(st, ((M + NB - 1) / NB) * NB * NB);
  GPGP_CUDA(cudaMemcpyAsync(Lm.p, Cm.p, M * M * sizeof(double), cudaMemcpyDeviceToDevice, st));
  double ldm = 0.0;
  if (chol_small(ctx, Lm.p, M, Wm.p, &ldm) != 0) {
    *failed = true;
    return GPGP_OK;
  }
  lS.alloc(st, ng);
  log_vec2_kernel<<<g1(ng), 256, 0, st>>>(ng, Sg.p, lS.p);
  GPGP_CHECK_LAUNCH();
  const double logdet_g = red.sum(lS.p, ng, 4) - 2.0 * logdet_z + 2.0 * ldm;
  // alpha1 = z / S - iDU C_m^-1 (iDU^T z); f1 = U K_z^-1 (U^T alpha1) + D alpha1
  a1.alloc(st, ng);
  t.alloc(st, M);
  q.alloc(st, ng);
  fg.alloc(st, ng);
  gemv64(st, true, ng, M, 1.0, iDUg.p, ng, zg.p, 0.0, t.p);
  tri_vec(st, Lm.p, M, M, t.p, t.p, false);
  tri_vec(st, Lm.p, M, M, t.p, t.p, true);
  gemv64(st, false, ng, M, 1.0, iDUg.p, ng, t.p, 0.0, q.p);
  div_vec_kernel<<<g1(ng), 256, 0, st>>>(ng, zg.p, Sg.p, a1.p);
  GPGP_CHECK_LAUNCH();
  vec_axpby(st, ng, -1.0, q.p, 1.0, a1.p);
  gemv64(st, true, ng, M, 1.0, Ug.p, ng, a1.p, 0.0, t.p);
  tri_vec(st, f.Lz.p, M, M, t.p, t.p, false);
  tri_vec(st, f.Lz.p, M, M, t.p, t.p, true);
  gemv64(st, false, ng, M, 1.0, Ug.p, ng, t.p, 0.0, q.p);
  fma_vec_kernel<<<g1(ng), 256, 0, st>>>(ng, q.p, Dg.p, a1.p, fg.p);
  GPGP_CHECK_LAUNCH();
  double lml1, lpu1 = 0.0;
  if (!ep) {
    lik_loglik(st, m->lk, ng, fg.p, yg.p, trials ? tg.p : nullptr, offset ? og.p : nullptr, red.b.p + 400,
               red.b.p + 200);
    const double ll = read_scalar(ctx, red.b.p + 400);
    const double fa = red.dot(fg.p, a1.p, ng);
    log_vec2_kernel<<<g1(ng), 256, 0, st>>>(ng, Vg.p, lS.p);
    GPGP_CHECK_LAUNCH();
    const double slogV = red.sum(lS.p, ng, 5);
    lml1 = ll - 0.5 * fa + 0.5 * (slogV - logdet_g);
    lpu1 = ll - 0.5 * fa;
  } else {
    DBuf terms, tg2;
    terms.alloc(st, n);
    ep_terms2_kernel<<<g1(n), 256, 0, st>>>(n, logC, m->cav_var.p, m->cav_mean.p, m->z.p, m->V.p, terms.p);
    GPGP_CHECK_LAUNCH();
    gat(tg2, terms.p, n, 1, good, ng);
    lml1 = -0.5 * logdet_g - 0.5 * red.dot(zg.p, a1.p, ng) + red.sum(tg2.p, ng, 6);
  }
  // the bad sites' prior given the good ones
  DBuf K21, pm, pc, Q, Qc;
  K21.alloc(st, nb * ng);
  gemm64(st, false, true, nb, ng, M, 1.0, Xb.p, nb, Xg.p, ng, 0.0, K21.p, nb);
  pm.alloc(st, nb);
  gemv64(st, false, nb, ng, 1.0, K21.p, nb, a1.p, 0.0, pm.p);
  // K21 inv_lemma_solve(C_inv, K21^T) = K21 S^-1 K21^T - (K21 iDU) C_m^-1 (K21 iDU)^T
  Q.alloc(st, nb * M);
  gemm64(st, false, false, nb, M, ng, 1.0, K21.p, nb, iDUg.p, ng, 0.0, Q.p, nb);
  Qc.alloc(st, nb * M);
  tri_rows(st, Lm.p, M, M, Q.p, nb, Qc.p, nb, nb, 0);
  tri_rows(st, Lm.p, M, M, Qc.p, nb, Qc.p, nb, nb, 1);
  pc.alloc(st, nb * nb);
  gemm64(st, false, true, nb, nb, M, 1.0, Xb.p, nb, Xb.p, nb, 0.0, pc.p, nb);  // X_bad X_bad^T
  {
    DBuf KS;
    KS.alloc(st, nb * ng);
    GPGP_CUDA(cudaMemcpyAsync(KS.p, K21.p, nb * ng * sizeof(double), cudaMemcpyDeviceToDevice, st));
    DBuf iS;
    iS.alloc(st, ng);
    recip2_kernel<<<g1(ng), 256, 0, st>>>(ng, Sg.p, iS.p);
    GPGP_CHECK_LAUNCH();
    scale_cols_kernel<<<gs(nb * ng), 256, 0, st>>>(nb, ng, KS.p, iS.p);  // K21 S^-1
    GPGP_CHECK_LAUNCH();
    gemm64(st, false, true, nb, nb, ng, -1.0, KS.p, nb, K21.p, nb, 1.0, pc.p, nb);
  }
  gemm64(st, false, true, nb, nb, M, 1.0, Q.p, nb, Qc.p, nb, 1.0, pc.p, nb);
  {
    DBuf dd;
    dd.alloc(st, nb);
    GPGP_CUDA(cudaMemcpyAsync(dd.p, Db.p, nb * sizeof(double), cudaMemcpyDeviceToDevice, st));
    add_diag2_kernel<<<g1(nb), 256, 0, st>>>(pc.p, nb, dd.p);
    GPGP_CHECK_LAUNCH();
  }
  double lml2 = 0.0, lpu2 = 0.0;
  gpgp_status s2 = nlc_bad_terms(m, nb, bad.p, pm.p, pc.p, zb.p, Vb.p, yb.p, trials ? tb.p : nullptr,
                                 offset ? ob.p : nullptr, ep, logC, &lml2, &lpu2, improper);
  if (s2 != GPGP_OK) {
    // chol(pred_cov) failing is an R error inside the reference's tryCatch: -Inf
    *failed = true;
    return GPGP_OK;
  }
  *lml = lml1 + lml2;
  *lpu = lpu1 + lpu2;
  return GPGP_OK;
}

}  // namespace

// ---------------------------------------------------------------------------
gpgp_status fit_fitc(gpgp_model *m, gpgp_fit_result *res, const double *inducing, bool on_device) {
  gpgp_ctx *ctx = m->ctx;
  cudaStream_t st = ctx->stream;
  const int64_t n = m->n;
  const int64_t M = m->method.num_inducing;
  if (M < 1 || !inducing) return fail(ctx, GPGP_EINVAL, "method_fitc needs inducing points");
  m->fitc.reset(new FitcState());
  FitcState &f = *m->fitc;
  f.M = M;
  const double *trials = m->has_trials ? m->trials.p : nullptr;
  const double *offset = m->has_offset ? m->offset.p : nullptr;
  const double jit = m->opts.jitter;
  Red red(ctx);
  res->iters = 0;
  res->converged = 1;
  res->quad_ok = 1;
  res->info = 0;
  // ---- set-up (R/gp_fit.R:104-111) ----
  copy_in(st, f.z, inducing, (size_t)M * m->d, on_device);
  f.Fz.alloc(st, (size_t)M * std::max(1, m->dk.nfeat));
  prep_features(st, m->dk, m->prep, f.z.p, M, M, f.Fz.p, M);
  f.Kz.alloc(st, (size_t)M * M);
  f.Lz.alloc(st, (size_t)M * M);
  f.Wz_blk.alloc(st, (size_t)((M + NB - 1) / NB) * NB * NB);
  f.Kxz.alloc(st, (size_t)n * M);
  f.X.alloc(st, (size_t)n * M);
  f.D.alloc(st, n);
  f.Kdiag.alloc(st, n);
  f.S.alloc(st, n);
  f.iDU.alloc(st, (size_t)n * M);
  f.Cm.alloc(st, (size_t)M * M);
  f.Lm.alloc(st, (size_t)M * M);
  f.Wm_blk.alloc(st, (size_t)((M + NB - 1) / NB) * NB * NB);
  {
    Phase ph(ctx, GPGP_PHASE_COV);
    cov_matrix(st, m->dk, 0xffffffffu, f.Fz.p, M, M, f.Fz.p, M, M, f.Kz.p, M, COV_FULL, 1, 1, jit, nullptr);
    cov_matrix(st, m->dk, 0xffffffffu, m->F.p, n, n, f.Fz.p, M, M, f.Kxz.p, n, COV_FULL, 0, 0, 0.0, nullptr);
    cov_diag(st, m->dk, 0xffffffffu, m->F.p, n, m->F.p, n, n, f.Kdiag.p);
  }
  GPGP_CUDA(cudaMemcpyAsync(f.Lz.p, f.Kz.p, M * M * sizeof(double), cudaMemcpyDeviceToDevice, st));
  double logdet_z = 0.0;
  // the reference wraps the FITC fit in tryCatch: a failed chol gives log_evidence -Inf
  auto minus_inf = [&](gpgp_status why) {
    m->log_evidence = -INFINITY;
    res->log_evidence = -INFINITY;
    res->status = why;
    m->fitted = 1;
    return GPGP_OK;
  };
  if (chol_small(ctx, f.Lz.p, M, f.Wz_blk.p, &logdet_z) != 0) return minus_inf(GPGP_ENOT_PD);
  {
    Phase ph(ctx, GPGP_PHASE_SOLVE);
    // X = Kxz Lz^-T, the transpose of forwardsolve(Kz_chol, t(Kxz)) (R/gp_fit.R:110)
    tri_rows(st, f.Lz.p, M, M, f.Kxz.p, n, f.X.p, n, n, 0);
  }
  // D = (diag K(x, x) + jitter) - colSums(forwardsolve(...)^2)  (R/gp_fit.R:109-110)
  {
    DBuf cs;
    cs.alloc(st, n);
    rowdot_nn_kernel<<<g1(n), 256, 0, st>>>(M, n, f.X.p, f.X.p, cs.p);
    GPGP_CHECK_LAUNCH();
    fitc_d_kernel<<<g1(n), 256, 0, st>>>(n, f.Kdiag.p, jit, cs.p, f.D.p);
    GPGP_CHECK_LAUNCH();
  }
  m->alpha.alloc(st, n);
  m->fmean.alloc(st, n);
  m->z.alloc(st, n);
  m->V.alloc(st, n);
  IBuf flags;
  flags.alloc(st, 1);
  DBuf fnew, lV, tmpn;
  fnew.alloc(st, n);
  lV.alloc(st, n);
  tmpn.alloc(st, n);
  if (m->approx.kind == GPGP_APPROX_LAPLACE) {
    // ---- Laplace (R/laplace.R:299-325) ----
    const int maxiter = m->lik.kind == GPGP_LIK_GAUSSIAN ? 1 : std::max(1, m->approx.maxiter);
    GPGP_CUDA(cudaMemsetAsync(m->fmean.p, 0, n * sizeof(double), st));
    double old = -INFINITY, diff = 0.0, lml = 0.0;
    int it = 0;
    for (it = 1; it <= maxiter; ++it) {
      lik_pseudodata_la(st, m->lk, n, m->fmean.p, m->y.p, trials, offset, m->z.p, m->V.p);
      GPGP_CUDA(cudaMemsetAsync(flags.p, 0, sizeof(int), st));
      check_positive2_kernel<<<g1(n), 256, 0, st>>>(n, m->V.p, flags.p);
      GPGP_CHECK_LAUNCH();
      int hf = 0;
      GPGP_CUDA(cudaMemcpyAsync(&hf, flags.p, sizeof(int), cudaMemcpyDeviceToHost, st));
      GPGP_CUDA(cudaStreamSynchronize(st));
      if (hf & 2) return minus_inf(GPGP_ENAN);  // NA in all(V > 0): an R error, caught by tryCatch
      double nlc_lml = 0.0, nlc_lpu = 0.0;
      if (hf & 4) {
        // some pseudo-variance <= 0: the good / bad split (R/laplace.R:151-231)
        bool improper = false, failed = false;
        gpgp_status s2 = fitc_nlc_terms(m, red, logdet_z, false, nullptr, &nlc_lml, &nlc_lpu, &improper, &failed);
        if (s2 != GPGP_OK) return s2;
        // chol(A) failing returns no log_post_unnorm, on which R's loop then errors: -Inf
        if (failed || improper) return minus_inf(GPGP_ENOT_PD);
      }
      axpy_vec_kernel<<<g1(n), 256, 0, st>>>(n, f.D.p, 1.0, m->V.p, f.S.p);  // S = D + V
      GPGP_CHECK_LAUNCH();
      if (!lemma_get(m, red, logdet_z)) return minus_inf(GPGP_ENOT_PD);
      lemma_solve_vec(m, m->z.p, m->alpha.p);
      fitc_fmean(m, m->alpha.p, fnew.p);
      double lpu;
      if (hf & 4) {
        lml = nlc_lml;
        lpu = nlc_lpu;
      } else {
        lik_loglik(st, m->lk, n, fnew.p, m->y.p, trials, offset, red.b.p + 400, red.b.p + 200);
        const double ll = read_scalar(ctx, red.b.p + 400);
        const double fa = red.dot(fnew.p, m->alpha.p, n);
        log_vec2_kernel<<<g1(n), 256, 0, st>>>(n, m->V.p, lV.p);
        GPGP_CHECK_LAUNCH();
        const double slogV = red.sum(lV.p, n, 2);
        lml = ll - 0.5 * fa + 0.5 * (slogV - f.logdet);
        lpu = ll - 0.5 * fa;
      }
      GPGP_CUDA(cudaMemcpyAsync(m->fmean.p, fnew.p, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
      diff = lpu - old;
      old = lpu;
      if (fabs(diff) < m->approx.tol) break;
    }
    if (it > maxiter) it = maxiter;
    res->iters = it;
    if (maxiter > 1 && it == maxiter && !(fabs(diff) < m->approx.tol)) res->converged = 0;
    m->log_evidence = lml;
    res->log_evidence = lml;
    res->status = GPGP_OK;
    m->fitted = 1;
    return GPGP_OK;
  }
  // ---- EP (R/ep.R:333-374) ----
  const int q = m->approx.quad_order;
  if (q < 1 || q > 64) return fail(ctx, GPGP_EINVAL, "quad_order must be in 1..64");
  std::vector<double> hx, hw;
  gauss_hermite(q, &hx, &hw);
  DBuf ghx, ghw, fm_old, fv_old, z_old, P_old, logC, terms;
  copy_in(st, ghx, hx.data(), q, false);
  copy_in(st, ghw, hw.data(), q, false);
  fm_old.alloc(st, n);
  fv_old.alloc(st, n);
  z_old.alloc(st, n);
  P_old.alloc(st, n);
  logC.alloc(st, n);
  terms.alloc(st, n);
  m->fvar.alloc(st, n);
  m->cav_mean.alloc(st, n);
  m->cav_var.alloc(st, n);
  GPGP_CUDA(cudaMemsetAsync(fm_old.p, 0, n * sizeof(double), st));
  GPGP_CUDA(cudaMemsetAsync(z_old.p, 0, n * sizeof(double), st));
  GPGP_CUDA(cudaMemsetAsync(P_old.p, 0, n * sizeof(double), st));
  // fvar_old = K_diag = diag K(x, x) + jitter (R/gp_fit.R:171, R/ep.R:342)
  fitc_d_kernel<<<g1(n), 256, 0, st>>>(n, f.Kdiag.p, jit, nullptr, fv_old.p);
  GPGP_CHECK_LAUNCH();
  // Y = X Lz^-1: the transpose of inv_Kz_Kzx = backsolve(t(Kz_chol), forwardsolve(Kz_chol, t(Kxz)))
  DBuf Y, VU, Qt, lhsU, auxT, d1, d2;
  Y.alloc(st, (size_t)n * M);
  tri_rows(st, f.Lz.p, M, M, f.X.p, n, Y.p, n, n, 1);
  VU.alloc(st, (size_t)n * M);
  Qt.alloc(st, (size_t)n * M);
  lhsU.alloc(st, (size_t)M * M);
  auxT.alloc(st, (size_t)n * M);
  d1.alloc(st, n);
  d2.alloc(st, n);
  const int maxiter = std::max(1, m->approx.maxiter);
  double diff_old = INFINITY, diff_new = INFINITY, damp = m->approx.damping, lml = -INFINITY;
  int it = 0, last_flags = 0;
  for (it = 1; it <= maxiter; ++it) {
    GPGP_CUDA(cudaMemsetAsync(flags.p, 0, sizeof(int), st));
    lik_ep_sites(st, m->lk, n, q, ghx.p, ghw.p, fm_old.p, fv_old.p, z_old.p, P_old.p, m->y.p, trials,
                 offset, damp, m->z.p, m->V.p, logC.p, m->cav_mean.p, m->cav_var.p, flags.p);
    int hf = 0;
    GPGP_CUDA(cudaMemcpyAsync(&hf, flags.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    GPGP_CUDA(cudaStreamSynchronize(st));
    last_flags = hf;
    if (hf & 2) {
      res->iters = it;
      res->quad_ok = (hf & 1) ? 0 : 1;
      GPGP_CUDA(cudaMemcpyAsync(m->fmean.p, fm_old.p, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
      return minus_inf(GPGP_ENAN);
    }
    double nlc_lml = 0.0;
    if (hf & 4) {
      // some site variance <= 0: the good / bad split (R/ep.R:186-272)
      bool improper = false, failed = false;
      double lpu_unused = 0.0;
      gpgp_status s2 = fitc_nlc_terms(m, red, logdet_z, true, logC.p, &nlc_lml, &lpu_unused, &improper, &failed);
      if (s2 != GPGP_OK) return s2;
      if (failed) return minus_inf(GPGP_ENOT_PD);
      if (improper) {
        // R returns fmean = Inf: the sweep is rejected after an accepted one; on the
        // first sweep R goes on without site variances and errors (tryCatch: -Inf)
        if (!(diff_old < INFINITY)) return minus_inf(GPGP_ENOT_PD);
        lml = -INFINITY;
        damp = damp * m->approx.damping;
        continue;
      }
    }
    axpy_vec_kernel<<<g1(n), 256, 0, st>>>(n, f.D.p, 1.0, m->V.p, f.S.p);
    GPGP_CHECK_LAUNCH();
    if (!lemma_get(m, red, logdet_z)) return minus_inf(GPGP_ENOT_PD);
    lemma_solve_vec(m, m->z.p, m->alpha.p);
    // fvar = diag1 + diag2 (R/ep.R:161-166), all in the transposed (n x M) form:
    // Q^T = diag(V) iDU C_m^-1, aux^T = diag(V/S) Y - Q^T (Y^T iDU)^T
    {
      scale_rows_kernel<<<gs(n * M), 256, 0, st>>>(n, M, f.iDU.p, m->V.p, VU.p);
      GPGP_CHECK_LAUNCH();
      rows_times_cminv(m, VU.p, Qt.p, n);
      gemm64(st, true, false, M, M, n, 1.0, Y.p, n, f.iDU.p, n, 0.0, lhsU.p, M);  // inv_Kz_Kzx iDU
      div_vec_kernel<<<g1(n), 256, 0, st>>>(n, m->V.p, f.S.p, tmpn.p);              // V / S
      GPGP_CHECK_LAUNCH();
      scale_rows_kernel<<<gs(n * M), 256, 0, st>>>(n, M, Y.p, tmpn.p, auxT.p);
      GPGP_CHECK_LAUNCH();
      gemm64(st, false, true, n, M, M, -1.0, Qt.p, n, lhsU.p, M, 1.0, auxT.p, n);
      rowdot_nn_kernel<<<g1(n), 256, 0, st>>>(M, n, f.Kxz.p, auxT.p, d1.p);          // diag1
      GPGP_CHECK_LAUNCH();
      rowdot_nn_kernel<<<g1(n), 256, 0, st>>>(M, n, f.iDU.p, Qt.p, d2.p);
      GPGP_CHECK_LAUNCH();
      // diag2 = D V / S - D * rowdot(iDU, Q^T)
      vec_mul(st, n, f.D.p, tmpn.p, lV.p);
      vec_mul(st, n, f.D.p, d2.p, d2.p);
      vec_axpby(st, n, 1.0, lV.p, -1.0, d2.p);
      vec_axpby(st, n, 1.0, d1.p, 1.0, d2.p);
      GPGP_CUDA(cudaMemcpyAsync(m->fvar.p, d2.p, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
    }
    fitc_fmean(m, m->alpha.p, m->fmean.p);
    ep_terms2_kernel<<<g1(n), 256, 0, st>>>(n, logC.p, m->cav_var.p, m->cav_mean.p, m->z.p, m->V.p,
                                             terms.p);
    GPGP_CHECK_LAUNCH();
    const double sterm = red.sum(terms.p, n, 3);
    const double za = red.dot(m->z.p, m->alpha.p, n);
    max_abs_diff(st, n, fm_old.p, m->fmean.p, red.b.p);
    diff_new = read_scalar(ctx, red.b.p + 64);
    lml = (hf & 4) ? nlc_lml : -0.5 * f.logdet - 0.5 * za + sterm;
    if (diff_new > diff_old) {
      damp = damp * m->approx.damping;
      continue;
    }
    damp = std::max(damp, m->approx.damping_min);
    GPGP_CUDA(cudaMemcpyAsync(fm_old.p, m->fmean.p, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
    GPGP_CUDA(cudaMemcpyAsync(fv_old.p, m->fvar.p, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
    GPGP_CUDA(cudaMemcpyAsync(z_old.p, m->z.p, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
    recip2_kernel<<<g1(n), 256, 0, st>>>(n, m->V.p, P_old.p);
    GPGP_CHECK_LAUNCH();
    diff_old = diff_new;
    if (diff_new < m->approx.tol) break;
  }
  if (it > maxiter) it = maxiter;
  res->iters = it;
  res->quad_ok = (last_flags & 1) ? 0 : 1;
  res->status = GPGP_OK;
  if (maxiter > 1 && it == maxiter) {
    lml = -INFINITY;
    res->converged = 0;
    res->status = GPGP_EMAXITER;
  }
  if (!res->quad_ok) lml = -INFINITY;
  m->log_evidence = lml;
  res->log_evidence = lml;
  m->fitted = 1;
  return GPGP_OK;
}

// ---------------------------------------------------------------------------
// caches independent of the test points: Sig1 = X^T S^-1 X (= A1 S^-1 A1^T),
// P = X^T iDU (= A1 iDU) and sol = Sig1 - P C_m^-1 P^T, the lemma solve
// inv_lemma_solve(C_inv, t(A1), A1) of R/gp_pred.R:271,283
static void fitc_pred_cache(gpgp_model *m) {
  FitcState &f = *m->fitc;
  if (f.have_pred_cache) return;
  cudaStream_t st = m->ctx->stream;
  const int64_t n = m->n, M = f.M;
  f.Sig1.alloc(st, (size_t)M * M);
  f.P.alloc(st, (size_t)M * M);
  DBuf XS, rs, Z;
  XS.alloc(st, (size_t)n * M);
  rs.alloc(st, n);
  recip2_kernel<<<g1(n), 256, 0, st>>>(n, f.S.p, rs.p);
  GPGP_CHECK_LAUNCH();
  scale_rows_kernel<<<gs(n * M), 256, 0, st>>>(n, M, f.X.p, rs.p, XS.p);
  GPGP_CHECK_LAUNCH();
  gemm64(st, true, false, M, M, n, 1.0, XS.p, n, f.X.p, n, 0.0, f.Sig1.p, M);
  gemm64(st, true, false, M, M, n, 1.0, f.X.p, n, f.iDU.p, n, 0.0, f.P.p, M);
  // Z = P C_m^-1 (rows of P), sol = Sig1 - Z P^T
  Z.alloc(st, (size_t)M * M);
  rows_times_cminv(m, f.P.p, Z.p, M);
  gemm64(st, false, true, M, M, M, -1.0, Z.p, M, f.P.p, M, 1.0, f.Sig1.p, M);  // Sig1 <- sol
  f.have_pred_cache = true;
}

gpgp_status pred_fitc(gpgp_model *m, const double *Ft, int64_t mt, uint32_t gm, double *mean,
                      double *var) {
  FitcState &f = *m->fitc;
  cudaStream_t st = m->ctx->stream;
  const int64_t n = m->n, M = f.M;
  DBuf Ktz, X2, v1;
  Ktz.alloc(st, (size_t)mt * M);
  X2.alloc(st, (size_t)mt * M);
  v1.alloc(st, M);
  cov_matrix(st, m->dk, gm, Ft, mt, mt, f.Fz.p, M, M, Ktz.p, mt, COV_FULL, 0, 0, 0.0, nullptr);
  tri_rows(st, f.Lz.p, M, M, Ktz.p, mt, X2.p, mt, mt, 0);        // X2 = Ktz Lz^-T (= Kt_aux2^T)
  gemv64(st, true, n, M, 1.0, f.X.p, n, m->alpha.p, 0.0, v1.p);  // Kt_aux1 alpha
  gemv64(st, false, mt, M, 1.0, X2.p, mt, v1.p, 0.0, mean);      // t(Kt_aux2) (Kt_aux1 alpha)
  if (!var) return GPGP_OK;
  // Dt = diag K(xt, xt) - colSums(Kt_aux2^2)
  DBuf Dt, cs, Y2, pv, auxT, red;
  Dt.alloc(st, mt);
  cs.alloc(st, mt);
  cov_diag(st, m->dk, gm, Ft, mt, Ft, mt, mt, Dt.p);
  rowdot_nn_kernel<<<g1(mt), 256, 0, st>>>(M, mt, X2.p, X2.p, cs.p);
  GPGP_CHECK_LAUNCH();
  vec_axpby(st, mt, -1.0, cs.p, 1.0, Dt.p);
  // prior_var = rowSums(Ktz * t(Kz^-1 Ktz^T)) + Dt, (Kz^-1 Ktz^T)^T = X2 Lz^-1
  Y2.alloc(st, (size_t)mt * M);
  tri_rows(st, f.Lz.p, M, M, X2.p, mt, Y2.p, mt, mt, 1);
  pv.alloc(st, mt);
  rowdot_nn_kernel<<<g1(mt), 256, 0, st>>>(M, mt, Ktz.p, Y2.p, pv.p);
  GPGP_CHECK_LAUNCH();
  vec_axpby(st, mt, 1.0, Dt.p, 1.0, pv.p);
  // var_reduction = colSums(Kt_aux2 * (sol Kt_aux2)) = rowdot(X2, X2 sol^T)
  fitc_pred_cache(m);
  auxT.alloc(st, (size_t)mt * M);
  gemm64(st, false, true, mt, M, M, 1.0, X2.p, mt, f.Sig1.p, M, 0.0, auxT.p, mt);
  red.alloc(st, mt);
  rowdot_nn_kernel<<<g1(mt), 256, 0, st>>>(M, mt, X2.p, auxT.p, red.p);
  GPGP_CHECK_LAUNCH();
  axpy_vec_kernel<<<g1(mt), 256, 0, st>>>(mt, pv.p, -1.0, red.p, var);
  GPGP_CHECK_LAUNCH();
  return GPGP_OK;
}

// Full predictive covariance of a FITC fit (gp_pred_post.method_fitc with cov = TRUE,
// R/gp_pred.R:263-276, test points apart from the training inputs):
//   prior_cov = A2^T A2 + diag(Dt),  A2 = Lz^-1 K(z, xt) (the rows of X2 = A2^T),
//   cov = prior_cov - A2^T sol A2 + jitter I,  sol = A1 C^-1 A1^T (the cached Sig1).
// Mean as in pred_fitc. C is mt x mt column-major (device).
gpgp_status pred_cov_fitc(gpgp_model *m, const double *Ft, int64_t mt, uint32_t gm, double jitter, double *mean,
                          double *C) {
  FitcState &f = *m->fitc;
  cudaStream_t st = m->ctx->stream;
  const int64_t n = m->n, M = f.M;
  DBuf Ktz, X2, v1, Dt, cs, T;
  Ktz.alloc(st, (size_t)mt * M);
  X2.alloc(st, (size_t)mt * M);
  v1.alloc(st, M);
  cov_matrix(st, m->dk, gm, Ft, mt, mt, f.Fz.p, M, M, Ktz.p, mt, COV_FULL, 0, 0, 0.0, nullptr);
  tri_rows(st, f.Lz.p, M, M, Ktz.p, mt, X2.p, mt, mt, 0);        // X2 = Ktz Lz^-T
  gemv64(st, true, n, M, 1.0, f.X.p, n, m->alpha.p, 0.0, v1.p);  // Kt_aux1 alpha
  gemv64(st, false, mt, M, 1.0, X2.p, mt, v1.p, 0.0, mean);
  // Dt = diag K(xt, xt) - colSums(Kt_aux2^2)
  Dt.alloc(st, mt);
  cs.alloc(st, mt);
  cov_diag(st, m->dk, gm, Ft, mt, Ft, mt, mt, Dt.p);
  rowdot_nn_kernel<<<g1(mt), 256, 0, st>>>(M, mt, X2.p, X2.p, cs.p);
  GPGP_CHECK_LAUNCH();
  vec_axpby(st, mt, -1.0, cs.p, 1.0, Dt.p);
  gemm64(st, false, true, mt, mt, M, 1.0, X2.p, mt, X2.p, mt, 0.0, C, mt);  // A2^T A2
  add_diag2_kernel<<<g1(mt), 256, 0, st>>>(C, mt, Dt.p);
  GPGP_CHECK_LAUNCH();
  fitc_pred_cache(m);
  T.alloc(st, (size_t)mt * M);
  gemm64(st, false, false, mt, M, M, 1.0, X2.p, mt, f.Sig1.p, M, 0.0, T.p, mt);  // A2^T sol
  gemm64(st, false, true, mt, mt, M, -1.0, T.p, mt, X2.p, mt, 1.0, C, mt);
  fill_kernel<<<g1(mt), 256, 0, st>>>(mt, jitter, cs.p);
  GPGP_CHECK_LAUNCH();
  add_diag2_kernel<<<g1(mt), 256, 0, st>>>(C, mt, cs.p);
  GPGP_CHECK_LAUNCH();
  return GPGP_OK;
}

// Training-point posterior (gp_pred_post.method_fitc with train = TRUE,
// R/gp_pred.R:262-290) turned into LOO moments (R/gp_loo.R:119-129).
gpgp_status loo_fitc_posteriors(gpgp_model *m, double *lmean, double *lvar) {
  FitcState &f = *m->fitc;
  cudaStream_t st = m->ctx->stream;
  const int64_t n = m->n, M = f.M;
  fitc_pred_cache(m);
  // Dt = diag K(x, x) - colSums(A1^2)  (no jitter in prediction)
  DBuf Dt, cs, Y, pv, auxT, CiU, iCP, d1, d2, d3, ds, t3;
  Dt.alloc(st, n);
  cs.alloc(st, n);
  rowdot_nn_kernel<<<g1(n), 256, 0, st>>>(M, n, f.X.p, f.X.p, cs.p);
  GPGP_CHECK_LAUNCH();
  axpy_vec_kernel<<<g1(n), 256, 0, st>>>(n, f.Kdiag.p, -1.0, cs.p, Dt.p);
  GPGP_CHECK_LAUNCH();
  // prior_var = rowSums(Kxz * (X Lz^-1)) + Dt
  Y.alloc(st, (size_t)n * M);
  tri_rows(st, f.Lz.p, M, M, f.X.p, n, Y.p, n, n, 1);
  pv.alloc(st, n);
  rowdot_nn_kernel<<<g1(n), 256, 0, st>>>(M, n, f.Kxz.p, Y.p, pv.p);
  GPGP_CHECK_LAUNCH();
  vec_axpby(st, n, 1.0, Dt.p, 1.0, pv.p);
  // CiU^T = iDU C_m^-1, iCP = CiU^T P^T (n x M)
  CiU.alloc(st, (size_t)n * M);
  rows_times_cminv(m, f.iDU.p, CiU.p, n);
  iCP.alloc(st, (size_t)n * M);
  gemm64(st, false, true, n, M, M, 1.0, CiU.p, n, f.P.p, M, 0.0, iCP.p, n);
  ds.alloc(st, n);
  div_vec_kernel<<<g1(n), 256, 0, st>>>(n, Dt.p, f.S.p, ds.p);  // Dt / S
  GPGP_CHECK_LAUNCH();
  // aux^T = X sol^T + diag(Dt/S) X - diag(Dt) iCP   (R/gp_pred.R:271-272)
  auxT.alloc(st, (size_t)n * M);
  scale_rows_kernel<<<gs(n * M), 256, 0, st>>>(n, M, f.X.p, ds.p, auxT.p);
  GPGP_CHECK_LAUNCH();
  gemm64(st, false, true, n, M, M, 1.0, f.X.p, n, f.Sig1.p, M, 1.0, auxT.p, n);
  DBuf DiCP;
  DiCP.alloc(st, (size_t)n * M);
  scale_rows_kernel<<<gs(n * M), 256, 0, st>>>(n, M, iCP.p, Dt.p, DiCP.p);
  GPGP_CHECK_LAUNCH();
  vec_axpby(st, (int64_t)n * M, -1.0, DiCP.p, 1.0, auxT.p);
  d1.alloc(st, n);
  rowdot_nn_kernel<<<g1(n), 256, 0, st>>>(M, n, f.X.p, auxT.p, d1.p);  // diag1
  GPGP_CHECK_LAUNCH();
  // diag2 = (Dt/S) colSums(A1^2) - Dt rowdot(iCP, X)   (R/gp_pred.R:273)
  d2.alloc(st, n);
  vec_mul(st, n, ds.p, cs.p, d2.p);
  DBuf rd;
  rd.alloc(st, n);
  rowdot_nn_kernel<<<g1(n), 256, 0, st>>>(M, n, iCP.p, f.X.p, rd.p);
  GPGP_CHECK_LAUNCH();
  vec_mul(st, n, Dt.p, rd.p, rd.p);
  vec_axpby(st, n, -1.0, rd.p, 1.0, d2.p);
  // diag3 = Dt^2 / S - Dt^2 rowdot(iDU, CiU^T)   (R/gp_pred.R:274)
  d3.alloc(st, n);
  rowdot_nn_kernel<<<g1(n), 256, 0, st>>>(M, n, f.iDU.p, CiU.p, d3.p);
  GPGP_CHECK_LAUNCH();
  t3.alloc(st, n);
  vec_mul(st, n, Dt.p, ds.p, t3.p);
  vec_mul(st, n, Dt.p, d3.p, d3.p);
  vec_mul(st, n, Dt.p, d3.p, d3.p);
  vec_axpby(st, n, 1.0, t3.p, -1.0, d3.p);
  // post_var = prior_var - (d1 + d2 + d3)
  vec_axpby(st, n, -1.0, d1.p, 1.0, pv.p);
  vec_axpby(st, n, -1.0, d2.p, 1.0, pv.p);
  vec_axpby(st, n, -1.0, d3.p, 1.0, pv.p);
  // LOO moments: loo_var = 1 / (1/post_var - 1/V), loo_mean = fhat - loo_var (z - fhat) / V
  loo_moments_kernel<<<g1(n), 256, 0, st>>>(n, pv.p, m->V.p, m->z.p, m->fmean.p, lmean, lvar);
  GPGP_CHECK_LAUNCH();
  return GPGP_OK;
}

}  // namespace gpgp
