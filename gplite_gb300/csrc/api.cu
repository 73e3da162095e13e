// C ABI of libgpgp: contexts, models, and the host-side orchestration of the
// GP hot path (fit / energy gradient / prediction / LOO) on one GPU.
//
// The iteration logic restates the reference's R loops: laplace.method_full
// (R/laplace.R:274-297), laplace_iter.method_full (R/laplace.R:13-39),
// ep.method_full (R/ep.R:286-330), ep_iter.method_full (R/ep.R:16-49),
// gp_pred_post.method_full (R/gp_pred.R:202-232) and loo_posteriors
// (R/gp_loo.R:119-133). All O(n^2) and O(n^3) work runs in the kernels of
// cov.cu / dense.cu / lik.cu; the host only sequences launches and reads back
// the few scalars the convergence tests need.
#include <math.h>

#include <algorithm>
#include <cstring>
#include <limits>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "common.cuh"
#include "model.cuh"

using namespace gpgp;

namespace gpgp {
thread_local std::string tl_error;
}

namespace {

// ---------------------------------------------------------------------------
// small elementwise kernels used only by the orchestration
// ---------------------------------------------------------------------------
__global__ void make_B_kernel(const double *__restrict__ K, int64_t n, const double *__restrict__ s,
                              double *__restrict__ B) {
  // B = I + diag(s) K diag(s), lower triangle (R/laplace.R:27: sqrt(1/V) * (K * sqrt(1/V)))
  for (int64_t j = blockIdx.y; j < n; j += gridDim.y) {
    for (int64_t i = j + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
      const double v = s[i] * (K[i + j * n] * s[j]);
      B[i + j * n] = (i == j) ? 1.0 + v : v;
    }
  }
}

__global__ void add_scalar_kernel(int64_t n, double a, double *__restrict__ v) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) v[i] += a;
}

__global__ void gauss_alpha_prep(int64_t n, const double *__restrict__ s, const double *__restrict__ z,
                                 double *__restrict__ t) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) t[i] = s[i] * z[i];
}

__global__ void check_positive_kernel(int64_t n, const double *__restrict__ V, int *flag) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    const double v = V[i];
    if (isnan(v)) atomicOr(flag, 2);
    else if (!(v > 0.0)) atomicOr(flag, 4);
  }
}

// fvar_i = V_i (1 - [B^-1]_ii)  (= V * diag(C^-1 K), R/ep.R:41)
__global__ void ep_fvar_kernel(int64_t n, const double *__restrict__ V,
                               const double *__restrict__ bdiag, double *__restrict__ fvar) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) fvar[i] = V[i] * (1.0 - bdiag[i]);
}

// per-site terms of the EP evidence (R/ep.R:45-46):
// out_i = logC_i + 0.5 log(vc_i + V_i) + 0.5 (mc_i - z_i)^2 / (vc_i + V_i)
__global__ void ep_site_terms_kernel(int64_t n, const double *__restrict__ logC,
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

__global__ void log_vec_kernel(int64_t n, const double *__restrict__ v, double *__restrict__ o) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) o[i] = log(v[i]);
}

__global__ void recip_kernel(int64_t n, const double *__restrict__ v, double *__restrict__ o) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) o[i] = 1.0 / v[i];
}

// LOO posteriors for approx_laplace (R/gp_loo.R:119-129) with the training-point
// posterior variance post_var_i = D_i - D_i^2 [B^-1]_ii / V_i, D_i = V_i + jitter
// (identical to diag(K - K C^-1 K) with C = K + jitter I + diag(V)).
__global__ void loo_laplace_kernel(int64_t n, double jitter, const double *__restrict__ fhat,
                                   const double *__restrict__ z, const double *__restrict__ V,
                                   const double *__restrict__ bdiag, double *__restrict__ lmean,
                                   double *__restrict__ lvar) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    const double Vi = V[i];
    const double D = Vi + jitter;
    const double pv = D - D * D * (bdiag[i] / Vi);
    const double grad = (z[i] - fhat[i]) / Vi;
    const double lv = 1.0 / (1.0 / pv - 1.0 / Vi);
    lvar[i] = lv;
    lmean[i] = fhat[i] - lv * grad;
  }
}

// LOO posteriors from the posterior variance pv at the training inputs
// (R/gp_loo.R:119-129); lvar holds pv on entry
__global__ void loo_from_pv_kernel(int64_t n, const double *__restrict__ fhat, const double *__restrict__ z,
                                   const double *__restrict__ V, double *__restrict__ lmean,
                                   double *__restrict__ lvar) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    const double Vi = V[i];
    const double grad = (z[i] - fhat[i]) / Vi;
    const double lv = 1.0 / (1.0 / lvar[i] - 1.0 / Vi);
    lvar[i] = lv;
    lmean[i] = fhat[i] - lv * grad;
  }
}

// W_ij = alpha_i alpha_j - s_i s_j Binv_ij on the lower triangle (in place)
__global__ void grad_w_kernel(int64_t n, const double *__restrict__ alpha,
                              const double *__restrict__ s, double *__restrict__ W) {
  for (int64_t j = blockIdx.y; j < n; j += gridDim.y)
    for (int64_t i = j + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
      W[i + j * n] = alpha[i] * alpha[j] - s[i] * s[j] * W[i + j * n];
}

__global__ void diag_scaled_kernel(int64_t n, const double *__restrict__ W,
                                   const double *__restrict__ s, double *__restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = W[i + i * n] * s[i] * s[i];
}

__global__ void sub_from_kernel(int64_t n, const double *__restrict__ a, double *__restrict__ b) {
  // b = a - b
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = a[i] - b[i];
}


__global__ void nonfinite_kernel(int64_t n, const double *__restrict__ v, int *__restrict__ flag) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    if (!isfinite(v[i])) atomicOr(flag, 1);
}

void make_B(cudaStream_t st, const double *K, int64_t n, const double *s, double *B) {
  dim3 g((unsigned)std::min<int64_t>((n + 255) / 256, 64), (unsigned)std::min<int64_t>(n, 65535));
  make_B_kernel<<<g, 256, 0, st>>>(K, n, s, B);
  GPGP_CHECK_LAUNCH();
}

// ---------------------------------------------------------------------------
// one B-factorisation: B = I + S K S, L = chol(B), alpha = S L^-T L^-1 S z,
// fnew = K alpha; returns 0 or the non-PD pivot
// ---------------------------------------------------------------------------
struct Work {
  DBuf K, t1, t2, u, rhs, red, logdet_part, ll_part, tmpv;
  IBuf status, flags;
};

// r = rhs - (u + s * Kalpha)
__global__ void refine_residual_kernel(int64_t n, const double *__restrict__ rhs,
                                       const double *__restrict__ u, const double *__restrict__ s,
                                       const double *__restrict__ Kalpha, double *__restrict__ r) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) r[i] = rhs[i] - (u[i] + s[i] * Kalpha[i]);
}

// FP64 iterative refinement in B-space on the current factor: r = s z - B u with
// B u = u + s (K alpha); u += B^-1 r; alpha = s u; fnew = K alpha. w.rhs holds s z
// and w.u the current solution.
// B^-1 b = L^-T (L^-1 b): by the flag-ordered triangular solves with L, or, once
// W = L^-1 is formed (m->Linv, use_w), by two triangular matrix-vector products.
void solve_B(gpgp_model *m, Work &w, const double *b, double *tmp, double *x, bool use_w) {
  cudaStream_t st = m->ctx->stream;
  const int64_t n = m->n;
  if (use_w) {
    trmv_lower(st, false, n, m->Linv.p, n, b, tmp);
    trmv_lower(st, true, n, m->Linv.p, n, tmp, x);
    return;
  }
  unsigned *bar = (unsigned *)w.flags.p + 2;
  trsv_flow(st, m->L.p, n, n, m->Winv.p, b, tmp, false, w.status.p, bar, m->errflag.p);
  trsv_flow(st, m->L.p, n, n, m->Winv.p, tmp, x, true, w.status.p, bar, m->errflag.p);
}

void refine_alpha(gpgp_model *m, Work &w, double *alpha, double *fnew, int iters, bool use_w = false) {
  cudaStream_t st = m->ctx->stream;
  const int64_t n = m->n;
  for (int it = 0; it < iters; ++it) {
    refine_residual_kernel<<<g1(n), 256, 0, st>>>(n, w.rhs.p, w.u.p, m->s.p, fnew, w.t1.p);
    GPGP_CHECK_LAUNCH();
    solve_B(m, w, w.t1.p, w.t2.p, w.t1.p, use_w);  // t1 <- B^-1 t1 (t1 -> t2 -> t1)
    vec_axpby(st, n, 1.0, w.t1.p, 1.0, w.u.p);
    vec_mul(st, n, m->s.p, w.u.p, alpha);
    gemv64(st, true, n, n, 1.0, w.K.p, n, alpha, 0.0, fnew);  // K symmetric: K alpha = K^T alpha
  }
}

// refine < 0: the model's own refinement count (mixed precision only). hflags
// (optional): w.flags[0] read back with the factorisation status in the same
// synchronisation; a set site flag (NaN or V <= 0) makes the result void, and no
// FP64 retry is made for it.
// hstatus_defer (optional, pinned host memory, FP64 only): the status and the
// flags (into hflags, pinned too) are copied without a synchronisation and 0 is
// returned; the caller reads both after its next one.
int64_t factor_and_solve(gpgp_model *m, Work &w, const double *zvec, double *alpha,
                         double *fnew, double *logdetL, bool force_fp64 = false, int refine = -1,
                         int *hflags = nullptr, int *hstatus_defer = nullptr) {
  gpgp_ctx *ctx = m->ctx;
  cudaStream_t st = ctx->stream;
  const int64_t n = m->n;
  GPGP_CUDA(cudaMemsetAsync(w.status.p, 0, sizeof(int), st));
  vec_rsqrt(st, n, m->V.p, m->s.p);
  if (m->b_ready && !force_fp64)
    m->b_ready = false;  // B was written with K by the covariance kernel
  else
    make_B(st, w.K.p, n, m->s.p, m->L.p);
  m->b_ready = false;
  const bool mixed = !force_fp64 && m->opts.precision == GPGP_PREC_MIXED;
  {
    Phase ph(ctx, GPGP_PHASE_POTRF);
    if (mixed)
      potrf_mixed(st, m->L.p, n, n, m->Winv.p, w.logdet_part.p, w.status.p, m->errflag.p, &ctx->side);
    else
      potrf(st, m->L.p, n, n, m->Winv.p, w.logdet_part.p, w.status.p, 1);
  }
  // When the energy gradient follows (mixed precision), W = L^-1, which it needs,
  // is formed now and the solves use it: two matrix-vector products in place of
  // the flag-ordered triangular solves, whose 64-row steps are serial.
  const bool use_w = mixed && m->want_linv;
  if (use_w) {
    Phase ph(ctx, GPGP_PHASE_TRTRI);
    if (m->Linv.n != (size_t)n * n) m->Linv.alloc(st, (size_t)n * n);
    trtri_mixed(st, m->L.p, n, n, m->Winv.p, m->Linv.p, n, m->errflag.p);
  }
  {
    Phase ph(ctx, GPGP_PHASE_SOLVE);
    // u = B^-1 (s z) with B = L L^T; alpha = s u
    gauss_alpha_prep<<<g1(n), 256, 0, st>>>(n, m->s.p, zvec, w.t1.p);
    GPGP_CHECK_LAUNCH();
    GPGP_CUDA(cudaMemcpyAsync(w.rhs.p, w.t1.p, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
    solve_B(m, w, w.t1.p, w.t2.p, w.u.p, use_w);
    vec_mul(st, n, m->s.p, w.u.p, alpha);
    gemv64(st, true, n, n, 1.0, w.K.p, n, alpha, 0.0, fnew);  // K symmetric: K alpha = K^T alpha
    if (mixed)
      refine_alpha(m, w, alpha, fnew, refine < 0 ? std::max(1, m->opts.refine_iters) : refine, use_w);
  }
  const int64_t nblk = (n + NB - 1) / NB;
  sum_vec(st, w.logdet_part.p, nblk, logdetL);
  if (hstatus_defer && !mixed) {
    GPGP_CUDA(cudaMemcpyAsync(hstatus_defer, w.status.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    if (hflags) GPGP_CUDA(cudaMemcpyAsync(hflags, w.flags.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    m->have_binv_diag = false;
    m->have_Linv = false;
    return 0;
  }
  int hstatus = 0;
  GPGP_CUDA(cudaMemcpyAsync(&hstatus, w.status.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  if (hflags) GPGP_CUDA(cudaMemcpyAsync(hflags, w.flags.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  GPGP_CUDA(cudaStreamSynchronize(st));
  m->have_binv_diag = false;
  m->have_Linv = use_w && hstatus == 0;
  if (hflags && (*hflags & 6)) return 0;
  if (hstatus != 0 && mixed) {
    // The sliced trailing updates carry an error of ~2^-33 of the largest entries
    // of B; when B's entries are large (big Laplace weights W) and a pivot is
    // small, that can break the factorisation of a matrix that is positive
    // definite in FP64. Redo this factorisation on the FP64 pipe, whose
    // verdict is the reference's.
    ++m->fp64_fallbacks;
    return factor_and_solve(m, w, zvec, alpha, fnew, logdetL, true, refine, hflags);
  }
  return hstatus;
}

// W = L^-1, kept on the model (FP64 blocked solve or the sliced recursive inverse).
void compute_linv(gpgp_model *m) {
  if (m->have_Linv) return;
  cudaStream_t st = m->ctx->stream;
  const int64_t n = m->n;
  if (m->Linv.n != (size_t)n * n) m->Linv.alloc(st, (size_t)n * n);
  Phase ph(m->ctx, GPGP_PHASE_TRTRI);
  if (m->opts.precision == GPGP_PREC_MIXED) {
    trtri_mixed(st, m->L.p, n, n, m->Winv.p, m->Linv.p, n, m->errflag.p);
  } else {
    DBuf tmp;
    tmp.alloc(st, (size_t)NB * n);
    IBuf status;
    status.alloc(st, 1);
    GPGP_CUDA(cudaMemsetAsync(status.p, 0, sizeof(int), st));
    trtri_lower(st, m->L.p, n, n, m->Winv.p, m->Linv.p, n, tmp.p, status.p);
  }
  m->have_Linv = true;
}

// diag(B^-1) = column sums of squares of L^-1.
void compute_binv_diag(gpgp_model *m) {
  cudaStream_t st = m->ctx->stream;
  const int64_t n = m->n;
  compute_linv(m);
  m->binv_diag.alloc(st, n);
  col_sumsq_lower(st, m->Linv.p, n, n, m->binv_diag.p);
  m->have_binv_diag = true;
}

// Reads the tensor-core error flag; a set flag means a bounded wait ran out.
bool tc_error(gpgp_model *m) {
  int h = 0;
  GPGP_CUDA(cudaMemcpyAsync(&h, m->errflag.p, sizeof(int), cudaMemcpyDeviceToHost, m->ctx->stream));
  GPGP_CUDA(cudaStreamSynchronize(m->ctx->stream));
  return h != 0;
}

gpgp_status fit_full(gpgp_model *m, gpgp_fit_result *res) {
  gpgp_ctx *ctx = m->ctx;
  cudaStream_t st = ctx->stream;
  const int64_t n = m->n;
  const double *trials = m->has_trials ? m->trials.p : nullptr;
  const double *offset = m->has_offset ? m->offset.p : nullptr;
  Work w;
  w.K.alloc(st, (size_t)n * n);
  w.t1.alloc(st, n);
  w.t2.alloc(st, n);
  w.u.alloc(st, n);
  w.rhs.alloc(st, n);
  w.red.alloc(st, 256);
  w.logdet_part.alloc(st, (n + NB - 1) / NB + 1);
  w.tmpv.alloc(st, n);
  w.status.alloc(st, 1);
  w.flags.alloc(st, 4 + (n + NB - 1) / NB);  // [0] site flags, [2..] ticket and block flags of the solves
  m->L.alloc(st, (size_t)n * n);
  m->Winv.alloc(st, (size_t)((n + NB - 1) / NB) * NB * NB);
  m->s.alloc(st, n);
  m->alpha.alloc(st, n);
  m->fmean.alloc(st, n);
  m->z.alloc(st, n);
  m->V.alloc(st, n);
  // K = eval_cf(x, x) + jitter I, stored in full (R/gp_fit.R:91-96). When the
  // energy gradient follows (gpgp_fit_grad), the same pass writes K's derivative
  // matrices, so the gradient does not evaluate the kernel a second time: for
  // matrices of at least as many 64-tiles as SMs, while they take at most half
  // of the free device memory.
  // Under mixed precision, kernels of stationary and constant terms are evaluated in
  // double-float arithmetic on the FP32 pipe (~2^-44 relative; the sliced
  // factorisation carries ~2^-33).
  {
    Phase ph(ctx, GPGP_PHASE_COV);
    m->dK.reset();
    m->have_dK = false;
    const bool df = m->opts.precision == GPGP_PREC_MIXED && n >= NB && cov_df_eligible(m->dk);
    // lik_gaussian (one factorisation, V = sigma^2): the covariance kernel also
    // writes B = I + K / sigma^2 into the factor's buffer, which the Cholesky
    // then starts from (factor_and_solve skips its own pass over K)
    const bool fuse_b = df && m->lik.kind == GPGP_LIK_GAUSSIAN && m->lik.sigma > 0.0 && m->approx.kind == GPGP_APPROX_LAPLACE;
    const double s2 = fuse_b ? 1.0 / (m->lik.sigma * m->lik.sigma) : 0.0;
    m->b_ready = false;
    const int64_t T = (n + NB - 1) / NB;
    if (m->want_dk && T * (T + 1) / 2 >= device_sms() && plan_grad_store(m->dk, &m->gplan) &&
        m->gplan.m.nmat > 0) {
      size_t fr = 0, tot = 0;
      GPGP_CUDA(cudaMemGetInfo(&fr, &tot));
      const size_t need = (size_t)m->gplan.m.nmat * n * n * sizeof(double);
      if (need <= fr / 2) {
        m->dK.alloc(st, (size_t)m->gplan.m.nmat * n * n);
        if (df)
          cov_matrix_df(st, m->dk, &m->gplan, m->F.p, n, n, w.K.p, n, m->opts.jitter, m->dK.p, n, n * n,
                        m->errflag.p, fuse_b ? m->L.p : nullptr, n, s2);
        else
          cov_matrix_grad(st, m->dk, m->gplan, m->F.p, n, n, w.K.p, n, m->opts.jitter, m->dK.p, n, n * n,
                          m->errflag.p);
        m->have_dK = true;
        m->b_ready = fuse_b;
      }
    }
    if (!m->have_dK) {
      if (df) {
        cov_matrix_df(st, m->dk, nullptr, m->F.p, n, n, w.K.p, n, m->opts.jitter, nullptr, 0, 0, m->errflag.p,
                      fuse_b ? m->L.p : nullptr, n, s2);
        m->b_ready = fuse_b;
      } else
        cov_matrix(st, m->dk, 0xffffffffu, m->F.p, n, n, m->F.p, n, n, w.K.p, n, COV_FULL, 1, 1,
                   m->opts.jitter, nullptr, m->errflag.p);
    }
  }
  double *red = w.red.p;  // [0..63] partials, [64] result, [100..] scalars
  double *logdetL = red + 100;
  res->iters = 0;
  res->converged = 1;
  res->quad_ok = 1;
  res->info = 0;
  if (m->approx.kind == GPGP_APPROX_LAPLACE) {
    int maxiter = m->lik.kind == GPGP_LIK_GAUSSIAN ? 1 : std::max(1, m->approx.maxiter);
    GPGP_CUDA(cudaMemsetAsync(m->fmean.p, 0, n * sizeof(double), st));
    DBuf fnew;
    fnew.alloc(st, n);
    double diff = 0.0;
    int it = 0;
    bool nlc_iter = false;  // the last iteration took the non-log-concave branch
    // FP64 Gaussian fit (one iteration, V = sigma^2 > 0): the factorisation's status
    // and site flags are read with the evidence terms, in one synchronisation
    const bool defer = m->opts.precision != GPGP_PREC_MIXED && maxiter == 1 &&
                       m->lik.kind == GPGP_LIK_GAUSSIAN && m->lik.sigma > 0.0;
    int *hdef = reinterpret_cast<int *>(ctx->h_pinned + 56);  // [0] status, [1] site flags
    hdef[0] = hdef[1] = 0;
    double nlc_lml = 0.0;
    for (it = 1; it <= maxiter; ++it) {
      lik_pseudodata_la(st, m->lk, n, m->fmean.p, m->y.p, trials, offset, m->z.p, m->V.p);
      GPGP_CUDA(cudaMemsetAsync(w.flags.p, 0, sizeof(int), st));
      check_positive_kernel<<<g1(n), 256, 0, st>>>(n, m->V.p, w.flags.p);
      GPGP_CHECK_LAUNCH();
      // mixed precision: the Newton iterates only steer the iteration, so their
      // solves go unrefined; the final alpha and f are refined once it stops
      const bool mixed = m->opts.precision == GPGP_PREC_MIXED;
      // The log-concave factorisation is queued before the site flags are read:
      // the flags come back with its status in one synchronisation, and a set
      // flag discards it.
      int hflags = 0;
      const int64_t info = factor_and_solve(m, w, m->z.p, m->alpha.p, fnew.p, logdetL, false,
                                            (mixed && maxiter > 1) ? 0 : -1, defer ? &hdef[1] : &hflags,
                                            defer ? &hdef[0] : nullptr);
      if (hflags & 2) {  // all(V > 0) is NA in R: an error
        res->status = GPGP_ENAN;
        res->log_evidence = NAN;
        return fail(ctx, GPGP_ENAN, "NaN in the Laplace pseudo-data");
      }
      if (hflags & 4) {
        // some pseudo-variance <= 0: the good / bad split (R/laplace.R:40-117), FP64
        bool improper = false;
        gpgp_status s2 = nlc_fit_full(m, w.K.p, nullptr, false, m->alpha.p, fnew.p, nullptr, &nlc_lml, &improper);
        if (s2 != GPGP_OK) {
          res->status = s2;
          res->log_evidence = -INFINITY;
          return s2;
        }
        if (improper)  // R returns fmean = fhat_old and -Inf
          GPGP_CUDA(cudaMemcpyAsync(fnew.p, m->fmean.p, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
        m->improper = improper;
        nlc_iter = true;
      } else {
        if (info != 0) {
          res->status = GPGP_ENOT_PD;
          res->info = info;
          res->log_evidence = -INFINITY;
          return fail(ctx, GPGP_ENOT_PD, "Cholesky factorisation: matrix is not positive definite");
        }
        m->nlc.reset();
        m->improper = false;
        nlc_iter = false;
      }
      if (maxiter > 1) {  // one iteration (lik_gaussian): the step size is not used
        max_abs_diff(st, n, m->fmean.p, fnew.p, red);
        diff = read_scalar(ctx, red + 64);
      }
      const bool last = diff < m->approx.tol || it == maxiter;
      if (last && mixed && maxiter > 1 && !nlc_iter)
        refine_alpha(m, w, m->alpha.p, fnew.p, std::max(1, m->opts.refine_iters));
      GPGP_CUDA(cudaMemcpyAsync(m->fmean.p, fnew.p, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
      if (diff < m->approx.tol) break;
    }
    if (it > maxiter) it = maxiter;
    res->iters = it;
    if (maxiter > 1 && it == maxiter && !(diff < m->approx.tol)) res->converged = 0;
    if (nlc_iter) {
      m->log_evidence = m->improper ? -INFINITY : nlc_lml;
    } else {
      // LML = loglik(f) - 0.5 f^T alpha - 0.5 (C_logdet - V_logdet), C_logdet - V_logdet = 2 sum log L_ii
      lik_loglik(st, m->lk, n, m->fmean.p, m->y.p, trials, offset, red + 101, red);
      dot_partial(st, n, m->fmean.p, m->alpha.p, red + 110);  // result at red + 174
      // red[100] (log det L), red[101] and red[174] in one copy
      double hr[75];
      GPGP_CUDA(cudaMemcpyAsync(hr, red + 100, sizeof(hr), cudaMemcpyDeviceToHost, st));
      GPGP_CUDA(cudaStreamSynchronize(st));
      if (defer) {
        if (hdef[1] & 6) {  // NaN sites (non-finite sigma or inputs)
          res->status = GPGP_ENAN;
          res->log_evidence = NAN;
          return fail(ctx, GPGP_ENAN, "NaN in the Laplace pseudo-data");
        }
        if (hdef[0] != 0) {
          res->status = GPGP_ENOT_PD;
          res->info = hdef[0];
          res->log_evidence = -INFINITY;
          return fail(ctx, GPGP_ENOT_PD, "Cholesky factorisation: matrix is not positive definite");
        }
      }
      const double ll = hr[1], fa = hr[74], ld = hr[0];
      m->log_evidence = ll - 0.5 * fa - 0.5 * (2.0 * ld);
    }
    res->log_evidence = m->log_evidence;
    res->status = GPGP_OK;
    return GPGP_OK;
  }
  // ---------------- EP (R/ep.R:286-330) ----------------
  const int q = m->approx.quad_order;
  if (q < 1 || q > 64) return fail(ctx, GPGP_EINVAL, "quad_order must be in 1..64");
  std::vector<double> hx, hw;
  gauss_hermite(q, &hx, &hw);
  DBuf ghx, ghw;
  copy_in(st, ghx, hx.data(), q, false);
  copy_in(st, ghw, hw.data(), q, false);
  DBuf fm_old, fv_old, z_old, P_old, logC, terms, fnew;
  fm_old.alloc(st, n);
  fv_old.alloc(st, n);
  z_old.alloc(st, n);
  P_old.alloc(st, n);
  logC.alloc(st, n);
  terms.alloc(st, n);
  fnew.alloc(st, n);
  m->fvar.alloc(st, n);
  m->cav_mean.alloc(st, n);
  m->cav_var.alloc(st, n);
  GPGP_CUDA(cudaMemsetAsync(fm_old.p, 0, n * sizeof(double), st));
  GPGP_CUDA(cudaMemsetAsync(z_old.p, 0, n * sizeof(double), st));
  GPGP_CUDA(cudaMemsetAsync(P_old.p, 0, n * sizeof(double), st));
  cov_diag(st, m->dk, 0xffffffffu, m->F.p, n, m->F.p, n, n, fv_old.p);
  // fvar_old = diag(K) with K = eval_cf(x, x) + jitter I (R/ep.R:295)
  add_scalar_kernel<<<g1(n), 256, 0, st>>>(n, m->opts.jitter, fv_old.p);
  GPGP_CHECK_LAUNCH();
  const int maxiter = std::max(1, m->approx.maxiter);
  const double tol = m->approx.tol;
  double diff_old = INFINITY, diff_new = INFINITY;
  double damp = m->approx.damping;
  int it = 0;
  int last_flags = 0;
  double lml = -INFINITY;
  for (it = 1; it <= maxiter; ++it) {
    GPGP_CUDA(cudaMemsetAsync(w.flags.p, 0, sizeof(int), st));
    lik_ep_sites(st, m->lk, n, q, ghx.p, ghw.p, fm_old.p, fv_old.p, z_old.p, P_old.p, m->y.p,
                 trials, offset, damp, m->z.p, m->V.p, logC.p, m->cav_mean.p, m->cav_var.p,
                 w.flags.p);
    int hflags = 0;
    GPGP_CUDA(cudaMemcpyAsync(&hflags, w.flags.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    GPGP_CUDA(cudaStreamSynchronize(st));
    last_flags = hflags;
    if (hflags & 2) {  // NA in sites (R/ep.R:30-32)
      res->iters = it;
      res->quad_ok = (hflags & 1) ? 0 : 1;
      res->status = GPGP_ENAN;
      m->log_evidence = -INFINITY;
      res->log_evidence = -INFINITY;
      GPGP_CUDA(cudaMemcpyAsync(m->fmean.p, fm_old.p, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
      m->fitted = 1;
      return GPGP_OK;
    }
    if (hflags & 4) {
      // some site variance <= 0: the good / bad split (R/ep.R:50-138), FP64
      bool improper = false;
      double lml_it = 0.0;
      gpgp_status s2 = nlc_fit_full(m, w.K.p, logC.p, true, m->alpha.p, fnew.p, m->fvar.p, &lml_it, &improper);
      if (s2 != GPGP_OK) {
        res->status = s2;
        return s2;
      }
      if (improper) {
        // R returns fmean = Inf: the sweep is rejected when an earlier one was
        // accepted; on the first sweep R goes on without site variances and errors
        if (!(diff_old < INFINITY)) {
          res->status = GPGP_ENOT_PD;
          return fail(ctx, GPGP_ENOT_PD, "EP: improper posterior of the bad sites in the first sweep");
        }
        m->improper = true;
        lml = -INFINITY;
        damp = damp * m->approx.damping;
        continue;
      }
      m->improper = false;
      GPGP_CUDA(cudaMemcpyAsync(m->fmean.p, fnew.p, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
      lml = lml_it;
      max_abs_diff(st, n, fm_old.p, m->fmean.p, red);
      diff_new = read_scalar(ctx, red + 64);
      if (diff_new > diff_old) {
        damp = damp * m->approx.damping;
        continue;
      }
      damp = std::max(damp, m->approx.damping_min);
      GPGP_CUDA(cudaMemcpyAsync(fm_old.p, m->fmean.p, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
      GPGP_CUDA(cudaMemcpyAsync(fv_old.p, m->fvar.p, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
      GPGP_CUDA(cudaMemcpyAsync(z_old.p, m->z.p, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
      recip_kernel<<<g1(n), 256, 0, st>>>(n, m->V.p, P_old.p);
      GPGP_CHECK_LAUNCH();
      diff_old = diff_new;
      if (diff_new < tol) break;
      continue;
    }
    m->nlc.reset();
    m->improper = false;
    int64_t info = factor_and_solve(m, w, m->z.p, m->alpha.p, fnew.p, logdetL);
    if (info != 0) {
      res->status = GPGP_ENOT_PD;
      res->info = info;
      return fail(ctx, GPGP_ENOT_PD, "Cholesky factorisation: matrix is not positive definite");
    }
    GPGP_CUDA(cudaMemcpyAsync(m->fmean.p, fnew.p, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
    compute_binv_diag(m);
    ep_fvar_kernel<<<g1(n), 256, 0, st>>>(n, m->V.p, m->binv_diag.p, m->fvar.p);
    GPGP_CHECK_LAUNCH();
    // evidence: -0.5 C_logdet - 0.5 z^T alpha + sum(site terms), C_logdet = 2 sum log L_ii + sum log V
    ep_site_terms_kernel<<<g1(n), 256, 0, st>>>(n, logC.p, m->cav_var.p, m->cav_mean.p, m->z.p,
                                                 m->V.p, terms.p);
    GPGP_CHECK_LAUNCH();
    sum_vec(st, terms.p, n, red + 102);
    log_vec_kernel<<<g1(n), 256, 0, st>>>(n, m->V.p, terms.p);
    GPGP_CHECK_LAUNCH();
    sum_vec(st, terms.p, n, red + 103);
    dot_partial(st, n, m->z.p, m->alpha.p, red + 110);
    max_abs_diff(st, n, fm_old.p, m->fmean.p, red);
    diff_new = read_scalar(ctx, red + 64);
    const double sterm = read_scalar(ctx, red + 102);
    const double slogV = read_scalar(ctx, red + 103);
    const double za = read_scalar(ctx, red + 174);
    const double ldL = read_scalar(ctx, logdetL);
    lml = -0.5 * (2.0 * ldL + slogV) - 0.5 * za + sterm;
    if (diff_new > diff_old) {
      damp = damp * m->approx.damping;
      continue;
    }
    damp = std::max(damp, m->approx.damping_min);
    GPGP_CUDA(cudaMemcpyAsync(fm_old.p, m->fmean.p, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
    GPGP_CUDA(cudaMemcpyAsync(fv_old.p, m->fvar.p, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
    GPGP_CUDA(cudaMemcpyAsync(z_old.p, m->z.p, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
    recip_kernel<<<g1(n), 256, 0, st>>>(n, m->V.p, P_old.p);
    GPGP_CHECK_LAUNCH();
    diff_old = diff_new;
    if (diff_new < tol) break;
  }
  if (it > maxiter) it = maxiter;
  res->iters = it;
  res->quad_ok = (last_flags & 1) ? 0 : 1;
  res->status = GPGP_OK;
  if (maxiter > 1 && it == maxiter) {  // R/ep.R:322-325
    lml = -INFINITY;
    res->converged = 0;
    res->status = GPGP_EMAXITER;
  }
  if (!res->quad_ok) lml = -INFINITY;  // R/ep.R:326-328
  m->log_evidence = lml;
  res->log_evidence = lml;
  return GPGP_OK;
}

gpgp_status fit_common(gpgp_ctx *ctx, const gpgp_kernel *k, const gpgp_lik *lik,
                       const gpgp_method *method, const gpgp_approx *approx,
                       const gpgp_fit_opts *opts, const double *x, int64_t n, int32_t d,
                       const double *y, const double *trials, const double *offset,
                       gpgp_model **model, gpgp_fit_result *result, bool on_device, bool want_grad = false) {
  if (!ctx || !k || !lik || !method || !approx || !opts || !x || !y || !model || !result)
    return fail(ctx, GPGP_EINVAL, "null argument");
  if (n < 1 || d < 1) return fail(ctx, GPGP_EINVAL, "n and d must be positive");
  std::memset(result, 0, sizeof(*result));
  *model = nullptr;
  if (lik->kind == GPGP_LIK_GAUSSIAN && approx->kind == GPGP_APPROX_EP)
    return fail(ctx, GPGP_EINVAL,
                "approx_ep disabled for lik_gaussian: use approx_laplace (R/gp.R:54-56)");
  if ((lik->kind == GPGP_LIK_BINOMIAL || lik->kind == GPGP_LIK_BETABINOM) && !trials)
    return fail(ctx, GPGP_EINVAL, "trials must be provided for the binomial and beta binomial likelihoods");
  if (lik->kind == GPGP_LIK_BETABINOM && !(lik->phi > 0))
    return fail(ctx, GPGP_EINVAL, "lik_betabinom needs phi > 0");
  if (method->kind < GPGP_METHOD_FULL || method->kind > GPGP_METHOD_RBF)
    return fail(ctx, GPGP_EINVAL, "unknown method");
  if (opts->precision != GPGP_PREC_FP64 && opts->precision != GPGP_PREC_MIXED)
    return fail(ctx, GPGP_EINVAL, "unknown precision");
  std::unique_ptr<gpgp_model> m(new gpgp_model());
  m->ctx = ctx;
  m->spec = *k;
  m->lik = *lik;
  m->lk = make_likdev(*lik);
  m->method = *method;
  m->approx = *approx;
  m->opts = *opts;
  m->n = n;
  m->d = d;
  std::string err;
  gpgp_status st = build_dev_kernel(k, d, &m->dk, &m->prep, &err);
  if (st != GPGP_OK) return fail(ctx, st, err);
  cudaStream_t s = ctx->stream;
  m->errflag.alloc(s, 1);
  GPGP_CUDA(cudaMemsetAsync(m->errflag.p, 0, sizeof(int), s));
  copy_in(s, m->x, x, (size_t)n * d, on_device);
  copy_in(s, m->y, y, n, on_device);
  // NaN or Inf in x or y: an error rather than NaN evidences. The flag travels to
  // pinned host memory with the fit and is read after the fit's next
  // synchronisation (the fit's result is discarded when it is set).
  IBuf bad;
  bad.alloc(s, 1);
  GPGP_CUDA(cudaMemsetAsync(bad.p, 0, sizeof(int), s));
  nonfinite_kernel<<<g1((int64_t)n * d), 256, 0, s>>>((int64_t)n * d, m->x.p, bad.p);
  GPGP_CHECK_LAUNCH();
  nonfinite_kernel<<<g1(n), 256, 0, s>>>(n, m->y.p, bad.p);
  GPGP_CHECK_LAUNCH();
  int *hflags = reinterpret_cast<int *>(ctx->h_pinned + 60);  // [0] inputs non-finite, [1] device wait timed out
  hflags[0] = 0;
  GPGP_CUDA(cudaMemcpyAsync(&hflags[0], bad.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  auto nan_inputs = [&]() -> gpgp_status {
    result->status = GPGP_ENAN;
    result->log_evidence = NAN;
    return fail(ctx, GPGP_ENAN, "x or y holds NaN or Inf");
  };
  if (trials) {
    copy_in(s, m->trials, trials, n, on_device);
    m->has_trials = true;
  }
  if (offset) {
    copy_in(s, m->offset, offset, n, on_device);
    m->has_offset = true;
  }
  m->F.alloc(s, (size_t)n * std::max(1, m->dk.nfeat));
  prep_features(s, m->dk, m->prep, m->x.p, n, n, m->F.p, n);
  if (method->kind == GPGP_METHOD_RF || method->kind == GPGP_METHOD_RBF) {
    // feature map of the reference's rf_featmap / rbf_featmap with the caller's draws
    m->rf.reset(new RfState());
    std::vector<double> hd;
    st = build_rf_spec(k, method, m->dk, &m->rf->spec, &hd, &err);
    if (st != GPGP_OK) return fail(ctx, st, err);
    m->rf->dr.alloc(s, std::max<size_t>(1, hd.size()));
    if (!hd.empty())
      GPGP_CUDA(cudaMemcpyAsync(m->rf->dr.p, hd.data(), hd.size() * sizeof(double), cudaMemcpyHostToDevice, s));
    // the caller's draws arrays may go once this call returns
    GPGP_CUDA(cudaStreamSynchronize(s));
    st = fit_rf(m.get(), result);
  } else if (method->kind == GPGP_METHOD_FITC) {
    st = fit_fitc(m.get(), result, method->inducing, on_device);
  } else {
    m->want_linv = want_grad && lik->kind == GPGP_LIK_GAUSSIAN && opts->precision == GPGP_PREC_MIXED;
    m->want_dk = want_grad && lik->kind == GPGP_LIK_GAUSSIAN;
    st = fit_full(m.get(), result);
  }
  if (st != GPGP_OK) {
    GPGP_CUDA(cudaStreamSynchronize(s));
    if (hflags[0]) return nan_inputs();
    return st;
  }
  hflags[1] = 0;
  GPGP_CUDA(cudaMemcpyAsync(&hflags[1], m->errflag.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  GPGP_CUDA(cudaStreamSynchronize(s));
  if (hflags[0]) return nan_inputs();
  if (hflags[1]) return fail(ctx, GPGP_ETIMEOUT, "a tensor-core kernel wait timed out");
  m->fitted = 1;
  *model = m.release();
  return GPGP_OK;
}

}  // namespace

// ===========================================================================
// exported functions
// ===========================================================================
extern "C" {

const char *gpgp_status_string(gpgp_status s) {
  switch (s) {
    case GPGP_OK: return "ok";
    case GPGP_ENOT_PD: return "matrix not positive definite";
    case GPGP_ENAN: return "NaN encountered";
    case GPGP_EMAXITER: return "maximum number of iterations reached";
    case GPGP_EUNSUPPORTED: return "unsupported";
    case GPGP_EOOM: return "out of device memory";
    case GPGP_ETIMEOUT: return "device wait timed out";
    case GPGP_ECUDA: return "CUDA error";
    case GPGP_EINVAL: return "invalid argument";
    case GPGP_ENOT_FITTED: return "model not fitted";
    case GPGP_EBUSY: return "busy";
  }
  return "unknown";
}

const char *gpgp_last_error(const gpgp_ctx *ctx) {
  return ctx ? ctx->last_error.c_str() : tl_error.c_str();
}

int64_t gpgp_launch_count(const gpgp_ctx *) { return g_launches; }

gpgp_status gpgp_create(gpgp_ctx **out, int device) {
  if (!out) return GPGP_EINVAL;
  *out = nullptr;
  std::unique_ptr<gpgp_ctx> c(new gpgp_ctx());
  gpgp_status st = guarded(nullptr, [&]() -> gpgp_status {
    int ndev = 0;
    GPGP_CUDA(cudaGetDeviceCount(&ndev));
    if (device < 0 || device >= ndev) return fail(nullptr, GPGP_EINVAL, "no such CUDA device");
    GPGP_CUDA(cudaSetDevice(device));
    c->device = device;
    {
      // keep up to a quarter of the device's memory in the pool between fits
      cudaMemPool_t pool;
      GPGP_CUDA(cudaDeviceGetDefaultMemPool(&pool, device));
      uint64_t cur = 0;
      GPGP_CUDA(cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &cur));
      size_t freeb = 0, total = 0;
      GPGP_CUDA(cudaMemGetInfo(&freeb, &total));
      uint64_t want = (uint64_t)total / 4;
      if (cur < want) GPGP_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &want));
    }
    GPGP_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    GPGP_CUDA(cudaStreamCreateWithFlags(&c->side.s, cudaStreamNonBlocking));
    GPGP_CUDA(cudaStreamCreateWithFlags(&c->side.s2, cudaStreamNonBlocking));
    for (cudaEvent_t *e : {&c->side.fork, &c->side.a, &c->side.l, &c->side.c, &c->side.b})
      GPGP_CUDA(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
    GPGP_CUDA(cudaMallocHost((void **)&c->h_pinned, 64 * sizeof(double)));
    return GPGP_OK;
  });
  if (st == GPGP_OK) *out = c.release();
  return st;
}

gpgp_status gpgp_destroy(gpgp_ctx *ctx) {
  if (!ctx) return GPGP_OK;
  cudaSetDevice(ctx->device);
  if (ctx->stream) {
    cudaStreamSynchronize(ctx->stream);
    cudaStreamDestroy(ctx->stream);
  }
  for (cudaStream_t x : {ctx->side.s, ctx->side.s2})
    if (x) {
      cudaStreamSynchronize(x);
      cudaStreamDestroy(x);
    }
  for (cudaEvent_t e : {ctx->side.fork, ctx->side.a, ctx->side.l, ctx->side.c, ctx->side.b})
    if (e) cudaEventDestroy(e);
  if (ctx->h_pinned) cudaFreeHost(ctx->h_pinned);
  delete ctx;
  return GPGP_OK;
}

gpgp_status gpgp_sync(gpgp_ctx *ctx) {
  if (!ctx) return GPGP_EINVAL;
  return guarded(ctx, [&]() -> gpgp_status {
    GPGP_CUDA(cudaStreamSynchronize(ctx->stream));
    return GPGP_OK;
  });
}

void *gpgp_stream(gpgp_ctx *ctx) { return ctx ? (void *)ctx->stream : nullptr; }

gpgp_status gpgp_profile_enable(gpgp_ctx *ctx, int32_t on) {
  if (!ctx) return GPGP_EINVAL;
  return guarded(ctx, [&]() -> gpgp_status {
    GPGP_CUDA(cudaSetDevice(ctx->device));
    prof_collect(ctx);
    for (int i = 0; i < GPGP_NPHASE; ++i) {
      ctx->prof_ms[i] = 0.0;
      ctx->prof_calls[i] = 0;
    }
    ctx->kt.reset();
    if (on < 0 || on > 2) return fail(ctx, GPGP_EINVAL, "gpgp_profile_enable: on must be 0, 1 or 2");
    ctx->prof = on != 0;
    ctx->prof_kernels = on == 1;
    return GPGP_OK;
  });
}

gpgp_status gpgp_kernel_profile_read(gpgp_ctx *ctx, int32_t kernel, int64_t *launches, double *ms,
                                     double *flops) {
  if (!ctx || kernel < 0 || kernel >= GPGP_NKPROF) return GPGP_EINVAL;
  return guarded(ctx, [&]() -> gpgp_status {
    GPGP_CUDA(cudaSetDevice(ctx->device));
    ctx->kt.collect();
    if (launches) *launches = ctx->kt.launches[kernel];
    if (ms) *ms = ctx->kt.ms[kernel];
    if (flops) *flops = ctx->kt.flops[kernel];
    return GPGP_OK;
  });
}

gpgp_status gpgp_profile_read(gpgp_ctx *ctx, double *ms, int64_t *calls) {
  if (!ctx) return GPGP_EINVAL;
  return guarded(ctx, [&]() -> gpgp_status {
    GPGP_CUDA(cudaSetDevice(ctx->device));
    prof_collect(ctx);
    for (int i = 0; i < GPGP_NPHASE; ++i) {
      if (ms) ms[i] = ctx->prof_ms[i];
      if (calls) calls[i] = ctx->prof_calls[i];
    }
    return GPGP_OK;
  });
}

gpgp_status gpgp_eval_cf(gpgp_ctx *ctx, const gpgp_kernel *k, const double *x1, int64_t n1,
                         const double *x2, int64_t n2, int32_t d, int32_t diag_only,
                         uint32_t group_mask, double *out) {
  if (!ctx || !k || !x1 || !x2 || !out || n1 < 0 || n2 < 0 || d < 1)
    return fail(ctx, GPGP_EINVAL, "invalid argument");
  return guarded(ctx, [&]() -> gpgp_status {
    GPGP_CUDA(cudaSetDevice(ctx->device));
    DevKernel dk;
    std::vector<HostTermPrep> prep;
    std::string err;
    gpgp_status st = build_dev_kernel(k, d, &dk, &prep, &err);
    if (st != GPGP_OK) return fail(ctx, st, err);
    cudaStream_t s = ctx->stream;
    const uint32_t gm = group_mask ? group_mask : 0xffffffffu;
    DBuf dx1, dx2, F1, F2, o;
    copy_in(s, dx1, x1, (size_t)n1 * d, false);
    copy_in(s, dx2, x2, (size_t)n2 * d, false);
    F1.alloc(s, (size_t)std::max<int64_t>(n1, 1) * dk.nfeat);
    F2.alloc(s, (size_t)std::max<int64_t>(n2, 1) * dk.nfeat);
    prep_features(s, dk, prep, dx1.p, n1, n1, F1.p, std::max<int64_t>(n1, 1));
    prep_features(s, dk, prep, dx2.p, n2, n2, F2.p, std::max<int64_t>(n2, 1));
    size_t cnt;
    if (diag_only) {
      const int64_t nd = std::min(n1, n2);
      cnt = nd;
      o.alloc(s, std::max<size_t>(cnt, 1));
      cov_diag(s, dk, gm, F1.p, std::max<int64_t>(n1, 1), F2.p, std::max<int64_t>(n2, 1), nd, o.p);
    } else {
      cnt = (size_t)n1 * n2;
      o.alloc(s, std::max<size_t>(cnt, 1));
      cov_matrix(s, dk, gm, F1.p, std::max<int64_t>(n1, 1), n1, F2.p, std::max<int64_t>(n2, 1), n2,
                 o.p, std::max<int64_t>(n1, 1), COV_FULL, 0, 0, 0.0, nullptr);
    }
    if (cnt) GPGP_CUDA(cudaMemcpyAsync(out, o.p, cnt * sizeof(double), cudaMemcpyDeviceToHost, s));
    GPGP_CUDA(cudaStreamSynchronize(s));
    return GPGP_OK;
  });
}

static gpgp_ctx *default_ctx(gpgp_status *st) {
  static std::mutex mu;
  static gpgp_ctx *ctx = nullptr;
  std::lock_guard<std::mutex> g(mu);
  if (!ctx) *st = gpgp_create(&ctx, 0);
  else *st = GPGP_OK;
  return ctx;
}

static gpgp_status one_term(int kind, const double *x1, int64_t n1, const double *x2, int64_t n2,
                            int32_t d, double lscale, double magn, double sigma0, double sigma,
                            int32_t diag_only, double *out) {
  gpgp_status st;
  gpgp_ctx *ctx = default_ctx(&st);
  if (st != GPGP_OK) return st;
  gpgp_kernel k;
  std::memset(&k, 0, sizeof(k));
  k.nterms = 1;
  k.ngroups = 1;
  k.term[0].kind = kind;
  k.term[0].lscale = lscale;
  k.term[0].magn = magn;
  k.term[0].sigma0 = sigma0;
  k.term[0].sigma = sigma;
  return gpgp_eval_cf(ctx, &k, x1, n1, x2, n2, d, diag_only, 0, out);
}

gpgp_status gpgp_cf_sexp(const double *x1, int64_t n1, const double *x2, int64_t n2, int32_t d,
                         double lscale, double magn, int32_t diag_only, double *out) {
  return one_term(GPGP_CF_SEXP, x1, n1, x2, n2, d, lscale, magn, 0, 0, diag_only, out);
}
gpgp_status gpgp_cf_matern32(const double *x1, int64_t n1, const double *x2, int64_t n2,
                             int32_t d, double lscale, double magn, int32_t diag_only,
                             double *out) {
  return one_term(GPGP_CF_MATERN32, x1, n1, x2, n2, d, lscale, magn, 0, 0, diag_only, out);
}
gpgp_status gpgp_cf_matern52(const double *x1, int64_t n1, const double *x2, int64_t n2,
                             int32_t d, double lscale, double magn, int32_t diag_only,
                             double *out) {
  return one_term(GPGP_CF_MATERN52, x1, n1, x2, n2, d, lscale, magn, 0, 0, diag_only, out);
}
gpgp_status gpgp_cf_nn(const double *x1, int64_t n1, const double *x2, int64_t n2, int32_t d,
                       double sigma0, double sigma, double magn, int32_t diag_only, double *out) {
  return one_term(GPGP_CF_NN, x1, n1, x2, n2, d, 1.0, magn, sigma0, sigma, diag_only, out);
}

// A mixed-precision Laplace / EP fit that breaks down (a pseudo-variance <= 0,
// NaN sites or quadrature) is redone in FP64, so that the mixed path never fails
// where the plain one would not: on the oscillating iterations that lead there
// the trajectories of the two precisions separate. A fit that merely reaches the
// iteration limit is returned as it is, flagged not converged, in either
// precision (the reference warns and returns its last iterate).
static gpgp_status fit_with_fallback(gpgp_ctx *ctx, const gpgp_kernel *k, const gpgp_lik *lik,
                                     const gpgp_method *method, const gpgp_approx *approx,
                                     const gpgp_fit_opts *opts, const double *x, int64_t n, int32_t d,
                                     const double *y, const double *trials, const double *offset,
                                     gpgp_model **model, gpgp_fit_result *result, bool on_device,
                                     bool want_grad = false) {
  gpgp_status st = fit_common(ctx, k, lik, method, approx, opts, x, n, d, y, trials, offset, model,
                              result, on_device, want_grad);
  const bool mixed = opts && opts->precision == GPGP_PREC_MIXED;
  if (result) result->precision_used = opts ? opts->precision : GPGP_PREC_FP64;
  if (!mixed || !lik || lik->kind == GPGP_LIK_GAUSSIAN) return st;
  const bool breakdown = st == GPGP_EUNSUPPORTED || st == GPGP_ENAN ||
                         (st == GPGP_OK && (result->status == GPGP_ENAN || result->status == GPGP_EUNSUPPORTED ||
                                            (approx && approx->kind == GPGP_APPROX_EP && !result->quad_ok)));
  if (!breakdown) return st;
  if (*model) {
    gpgp_model_free(*model);
    *model = nullptr;
  }
  gpgp_fit_opts o64 = *opts;
  o64.precision = GPGP_PREC_FP64;
  st = fit_common(ctx, k, lik, method, approx, &o64, x, n, d, y, trials, offset, model, result, on_device);
  result->precision_used = GPGP_PREC_FP64;
  return st;
}

// gp_fit and the energy gradient in one call; see include/gpgp.h.
static gpgp_status fit_grad_impl(gpgp_ctx *ctx, const gpgp_kernel *k, const gpgp_lik *lik,
                                 const gpgp_method *method, const gpgp_approx *approx,
                                 const gpgp_fit_opts *opts, const double *x, int64_t n, int32_t d,
                                 const double *y, const double *trials, const double *offset, gpgp_model **model,
                                 gpgp_fit_result *result, double *grad_terms, double *grad_lik_sigma,
                                 bool on_device) {
  if (!grad_terms) return fail(ctx, GPGP_EINVAL, "grad_terms is null");
  if (lik && method && (lik->kind != GPGP_LIK_GAUSSIAN || method->kind != GPGP_METHOD_FULL))
    return fail(ctx, GPGP_EUNSUPPORTED, "gradient needs lik_gaussian and method_full");
  gpgp_status st = guarded(ctx, [&]() {
    if (ctx) GPGP_CUDA(cudaSetDevice(ctx->device));
    return fit_with_fallback(ctx, k, lik, method, approx, opts, x, n, d, y, trials, offset, model, result,
                             on_device, true);
  });
  if (st != GPGP_OK) return st;
  return gpgp_model_grad(*model, grad_terms, grad_lik_sigma);
}

gpgp_status gpgp_fit_grad(gpgp_ctx *ctx, const gpgp_kernel *k, const gpgp_lik *lik, const gpgp_method *method,
                          const gpgp_approx *approx, const gpgp_fit_opts *opts, const double *x, int64_t n,
                          int32_t d, const double *y, const double *trials, const double *offset,
                          gpgp_model **model, gpgp_fit_result *result, double *grad_terms,
                          double *grad_lik_sigma) {
  return fit_grad_impl(ctx, k, lik, method, approx, opts, x, n, d, y, trials, offset, model, result, grad_terms,
                       grad_lik_sigma, false);
}

gpgp_status gpgp_fit_grad_dev(gpgp_ctx *ctx, const gpgp_kernel *k, const gpgp_lik *lik, const gpgp_method *method,
                              const gpgp_approx *approx, const gpgp_fit_opts *opts, const double *x, int64_t n,
                              int32_t d, const double *y, const double *trials, const double *offset,
                              gpgp_model **model, gpgp_fit_result *result, double *grad_terms,
                              double *grad_lik_sigma) {
  return fit_grad_impl(ctx, k, lik, method, approx, opts, x, n, d, y, trials, offset, model, result, grad_terms,
                       grad_lik_sigma, true);
}

gpgp_status gpgp_fit(gpgp_ctx *ctx, const gpgp_kernel *k, const gpgp_lik *lik,
                     const gpgp_method *method, const gpgp_approx *approx,
                     const gpgp_fit_opts *opts, const double *x, int64_t n, int32_t d,
                     const double *y, const double *trials, const double *offset,
                     gpgp_model **model, gpgp_fit_result *result) {
  return guarded(ctx, [&]() {
    if (ctx) GPGP_CUDA(cudaSetDevice(ctx->device));
    return fit_with_fallback(ctx, k, lik, method, approx, opts, x, n, d, y, trials, offset, model,
                             result, false);
  });
}

gpgp_status gpgp_fit_dev(gpgp_ctx *ctx, const gpgp_kernel *k, const gpgp_lik *lik,
                         const gpgp_method *method, const gpgp_approx *approx,
                         const gpgp_fit_opts *opts, const double *x, int64_t n, int32_t d,
                         const double *y, const double *trials, const double *offset,
                         gpgp_model **model, gpgp_fit_result *result) {
  return guarded(ctx, [&]() {
    if (ctx) GPGP_CUDA(cudaSetDevice(ctx->device));
    return fit_with_fallback(ctx, k, lik, method, approx, opts, x, n, d, y, trials, offset, model,
                             result, true);
  });
}

gpgp_status gpgp_model_free(gpgp_model *model) {
  if (!model) return GPGP_OK;
  cudaSetDevice(model->ctx->device);
  delete model;  // buffers are released on the context's stream
  return GPGP_OK;
}

gpgp_status gpgp_model_get(gpgp_model *m, int32_t field, double *out) {
  if (!m || !out) return GPGP_EINVAL;
  return guarded(m->ctx, [&]() -> gpgp_status {
    const double *src = nullptr;
    size_t count = m->n;
    if (field == GPGP_FIELD_WMEAN || field == GPGP_FIELD_WCOV) {
      if (!m->rf || !m->fitted) return fail(m->ctx, GPGP_EINVAL, "field not available for this model");
      const size_t D = m->rf->spec.D;
      src = field == GPGP_FIELD_WMEAN ? m->rf->wmean.p : m->rf->wcov.p;
      count = field == GPGP_FIELD_WMEAN ? D : D * D;
      GPGP_CUDA(cudaSetDevice(m->ctx->device));
      GPGP_CUDA(cudaMemcpyAsync(out, src, count * sizeof(double), cudaMemcpyDeviceToHost, m->ctx->stream));
      GPGP_CUDA(cudaStreamSynchronize(m->ctx->stream));
      return GPGP_OK;
    }
    switch (field) {
      case GPGP_FIELD_ALPHA: src = m->alpha.p; break;
      case GPGP_FIELD_FMEAN: src = m->fmean.p; break;
      case GPGP_FIELD_Z: src = m->z.p; break;
      case GPGP_FIELD_V: src = m->V.p; break;
      case GPGP_FIELD_FVAR: src = m->fvar.p; break;
      case GPGP_FIELD_CAVITY_MEAN: src = m->cav_mean.p; break;
      case GPGP_FIELD_CAVITY_VAR: src = m->cav_var.p; break;
      default: return fail(m->ctx, GPGP_EINVAL, "unknown field");
    }
    if (!src) return fail(m->ctx, GPGP_EINVAL, "field not available for this model");
    GPGP_CUDA(cudaSetDevice(m->ctx->device));
    GPGP_CUDA(cudaMemcpyAsync(out, src, m->n * sizeof(double), cudaMemcpyDeviceToHost,
                              m->ctx->stream));
    GPGP_CUDA(cudaStreamSynchronize(m->ctx->stream));
    return GPGP_OK;
  });
}

static gpgp_status pred_impl(gpgp_model *m, const double *xt, int64_t mt, uint32_t group_mask,
                             double *mean, double *var, bool on_device) {
  if (!m || !xt || !mean || mt < 0) return fail(m ? m->ctx : nullptr, GPGP_EINVAL, "invalid argument");
  if (!m->fitted) return fail(m->ctx, GPGP_ENOT_FITTED, "model is not fitted");
  if (m->improper)
    return fail(m->ctx, GPGP_ENOT_FITTED, "the fit has no posterior (log_evidence = -Inf, improper bad-site posterior)");
  gpgp_ctx *ctx = m->ctx;
  return guarded(ctx, [&]() -> gpgp_status {
    GPGP_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    const int64_t n = m->n;
    const uint32_t gm = group_mask ? group_mask : 0xffffffffu;
    if (mt == 0) return GPGP_OK;
    DBuf dxt, Ft, dmean;
    copy_in(s, dxt, xt, (size_t)mt * m->d, on_device);
    Ft.alloc(s, (size_t)mt * std::max(1, m->dk.nfeat));
    prep_features(s, m->dk, m->prep, dxt.p, mt, mt, Ft.p, mt);
    double *mout = mean;
    if (!on_device) {
      dmean.alloc(s, mt);
      mout = dmean.p;
    }
    if (m->fitc || m->rf) {
      DBuf dv;
      if (var) dv.alloc(s, mt);
      {
        Phase ph(ctx, GPGP_PHASE_PRED_VAR);
        gpgp_status st2 = m->rf ? pred_rf(m, Ft.p, mt, gm, mout, var ? dv.p : nullptr)
                                : pred_fitc(m, Ft.p, mt, gm, mout, var ? dv.p : nullptr);
        if (st2 != GPGP_OK) return st2;
      }
      if (var)
        GPGP_CUDA(cudaMemcpyAsync(var, dv.p, mt * sizeof(double),
                                  on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, s));
      if (!on_device)
        GPGP_CUDA(cudaMemcpyAsync(mean, mout, mt * sizeof(double), cudaMemcpyDeviceToHost, s));
      GPGP_CUDA(cudaStreamSynchronize(s));
      if (tc_error(m)) return fail(ctx, GPGP_ETIMEOUT, "a tensor-core kernel wait timed out");
      return GPGP_OK;
    }
    // mean = Kt alpha (R/gp_pred.R:209), fused: Kt is never stored. Mixed
    // precision evaluates the kernel in double-float arithmetic where it can.
    const bool df = m->opts.precision == GPGP_PREC_MIXED && cov_df_eligible(m->dk);
    {
      Phase ph(ctx, GPGP_PHASE_PRED_MEAN);
      if (df)
        cov_matvec_df(s, m->dk, gm, Ft.p, mt, mt, m->F.p, n, n, m->alpha.p, mout);
      else
        cov_matvec(s, m->dk, gm, Ft.p, mt, mt, m->F.p, n, n, m->alpha.p, mout);
    }
    if (var && m->nlc) {
      // a fit whose last iteration was non-log-concave: (K + V)^-1 through the blocks
      Phase ph(ctx, GPGP_PHASE_PRED_VAR);
      DBuf dv;
      dv.alloc(s, mt);
      nlc_pred_var(m, Ft.p, mt, gm, dv.p);
      GPGP_CUDA(cudaMemcpyAsync(var, dv.p, mt * sizeof(double),
                                on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, s));
    } else if (var) {
      Phase ph(ctx, GPGP_PHASE_PRED_VAR);
      // var = diag(Ktt) - colSums((C_chol^-1 Kt^T)^2), C_chol^-1 = L^-1 diag(s)  (R/gp_pred.R:216-228)
      const int64_t chunk = std::max<int64_t>(1, std::min<int64_t>(mt, (int64_t)(1ll << 28) / std::max<int64_t>(n, 1)));
      DBuf R, tmp, csum, kdiag;
      R.alloc(s, (size_t)n * chunk);
      tmp.alloc(s, (size_t)NB * chunk);
      csum.alloc(s, mt);
      kdiag.alloc(s, mt);
      IBuf status;
      status.alloc(s, 1);
      GPGP_CUDA(cudaMemsetAsync(status.p, 0, sizeof(int), s));
      const bool mixed = m->opts.precision == GPGP_PREC_MIXED;
      if (mixed) compute_linv(m);
      for (int64_t c0 = 0; c0 < mt; c0 += chunk) {
        const int64_t mc = std::min(chunk, mt - c0);
        if (df)
          cov_cross_df(s, m->dk, gm, m->F.p, n, n, Ft.p + c0, mt, mc, R.p, n, m->s.p);
        else
          cov_matrix(s, m->dk, gm, m->F.p, n, n, Ft.p + c0, mt, mc, R.p, n, COV_ROWSCALE, 0, 0, 0.0,
                     m->s.p);
        if (mixed) {
          trmv_sumsq_mixed(s, m->Linv.p, n, n, R.p, mc, n, csum.p + c0, m->errflag.p);
        } else {
          trsm_lower(s, m->L.p, n, n, m->Winv.p, R.p, mc, n, tmp.p, status.p);
          col_sumsq(s, R.p, n, mc, n, csum.p + c0);
        }
      }
      cov_diag(s, m->dk, gm, Ft.p, mt, Ft.p, mt, mt, kdiag.p);
      sub_from_kernel<<<g1(mt), 256, 0, s>>>(mt, kdiag.p, csum.p);
      GPGP_CHECK_LAUNCH();
      GPGP_CUDA(cudaMemcpyAsync(var, csum.p, mt * sizeof(double),
                                on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, s));
    }
    if (!on_device)
      GPGP_CUDA(cudaMemcpyAsync(mean, mout, mt * sizeof(double), cudaMemcpyDeviceToHost, s));
    GPGP_CUDA(cudaStreamSynchronize(s));
    if (tc_error(m)) return fail(ctx, GPGP_ETIMEOUT, "a tensor-core kernel wait timed out");
    return GPGP_OK;
  });
}

gpgp_status gpgp_pred(gpgp_model *m, const double *xt, int64_t mt, uint32_t group_mask,
                      double *mean, double *var) {
  return pred_impl(m, xt, mt, group_mask, mean, var, false);
}

gpgp_status gpgp_pred_dev(gpgp_model *m, const double *xt, int64_t mt, uint32_t group_mask,
                          double *mean, double *var) {
  return pred_impl(m, xt, mt, group_mask, mean, var, true);
}

// gp_loo (R/gp_loo.R:73-109): the LOO posteriors, then Gauss-Hermite quadrature of
// order quad_order (draws == 0) or Monte Carlo with the caller's standard normals z
// (n x draws, column-major: fsample = loo_mean + sd z, as R fills it).
static gpgp_status loo_impl(gpgp_model *m, int32_t quad_order, int64_t draws, const double *z, double *loos,
                            double *loo_sum) {
  if (!m || !loos) return fail(m ? m->ctx : nullptr, GPGP_EINVAL, "invalid argument");
  if (!m->fitted) return fail(m->ctx, GPGP_ENOT_FITTED, "model is not fitted");
  if (m->improper)
    return fail(m->ctx, GPGP_ENOT_FITTED, "the fit has no posterior (log_evidence = -Inf, improper bad-site posterior)");
  if (draws == 0 && (quad_order < 1 || quad_order > 64))
    return fail(m->ctx, GPGP_EINVAL, "quad_order must be in 1..64");
  if (draws < 0 || (draws > 0 && !z)) return fail(m->ctx, GPGP_EINVAL, "draws > 0 needs the normals z");
  gpgp_ctx *ctx = m->ctx;
  return guarded(ctx, [&]() -> gpgp_status {
    GPGP_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    const int64_t n = m->n;
    DBuf lmean, lvar, out, ghx, ghw, red;
    const double *mp, *vp;
    if (m->approx.kind == GPGP_APPROX_EP) {
      if (!m->cav_mean.p) return fail(ctx, GPGP_ENOT_FITTED, "EP fit has no cavity moments");
      mp = m->cav_mean.p;
      vp = m->cav_var.p;
    } else if (m->fitc) {
      lmean.alloc(s, n);
      lvar.alloc(s, n);
      gpgp_status st2 = loo_fitc_posteriors(m, lmean.p, lvar.p);
      if (st2 != GPGP_OK) return st2;
      mp = lmean.p;
      vp = lvar.p;
    } else if (m->rf) {
      // post_var = diag(Z wcov Z^T) at the training inputs (R/gp_loo.R:124, R/gp_pred.R:298-314)
      lmean.alloc(s, n);
      lvar.alloc(s, n);
      rf_train_var(m, lvar.p);
      loo_from_pv_kernel<<<g1(n), 256, 0, s>>>(n, m->fmean.p, m->z.p, m->V.p, lmean.p, lvar.p);
      GPGP_CHECK_LAUNCH();
      mp = lmean.p;
      vp = lvar.p;
    } else if (m->nlc) {
      // non-log-concave fit: post_var at the training inputs through the blocks of
      // (K + V)^-1 (gp_pred_post with train = TRUE, R/gp_loo.R:124)
      lmean.alloc(s, n);
      lvar.alloc(s, n);
      nlc_pred_var(m, m->F.p, n, 0xffffffffu, lvar.p);
      loo_from_pv_kernel<<<g1(n), 256, 0, s>>>(n, m->fmean.p, m->z.p, m->V.p, lmean.p, lvar.p);
      GPGP_CHECK_LAUNCH();
      mp = lmean.p;
      vp = lvar.p;
    } else {
      if (!m->have_binv_diag) compute_binv_diag(m);
      lmean.alloc(s, n);
      lvar.alloc(s, n);
      loo_laplace_kernel<<<g1(n), 256, 0, s>>>(n, m->opts.jitter, m->fmean.p, m->z.p, m->V.p,
                                               m->binv_diag.p, lmean.p, lvar.p);
      GPGP_CHECK_LAUNCH();
      mp = lmean.p;
      vp = lvar.p;
    }
    out.alloc(s, n);
    if (draws > 0) {
      DBuf dz;
      copy_in(s, dz, z, (size_t)n * draws, false);
      lik_loo_mc(s, m->lk, n, draws, dz.p, mp, vp, m->y.p, m->has_trials ? m->trials.p : nullptr,
                 m->has_offset ? m->offset.p : nullptr, out.p);
    } else {
      std::vector<double> hx, hw;
      gauss_hermite(quad_order, &hx, &hw);
      copy_in(s, ghx, hx.data(), quad_order, false);
      copy_in(s, ghw, hw.data(), quad_order, false);
      lik_loo_gh(s, m->lk, n, quad_order, ghx.p, ghw.p, mp, vp, m->y.p,
                 m->has_trials ? m->trials.p : nullptr, m->has_offset ? m->offset.p : nullptr, out.p);
    }
    GPGP_CUDA(cudaMemcpyAsync(loos, out.p, n * sizeof(double), cudaMemcpyDeviceToHost, s));
    GPGP_CUDA(cudaStreamSynchronize(s));
    if (loo_sum) {
      double acc = 0.0;
      for (int64_t i = 0; i < n; ++i) acc += loos[i];
      *loo_sum = acc;
    }
    return GPGP_OK;
  });
}

gpgp_status gpgp_loo(gpgp_model *m, int32_t quad_order, double *loos, double *loo_sum) {
  return loo_impl(m, quad_order, 0, nullptr, loos, loo_sum);
}

gpgp_status gpgp_loo_mc(gpgp_model *m, int64_t draws, const double *z, double *loos, double *loo_sum) {
  if (draws < 1) return fail(m ? m->ctx : nullptr, GPGP_EINVAL, "draws must be positive");
  return loo_impl(m, 0, draws, z, loos, loo_sum);
}

gpgp_status gpgp_model_grad(gpgp_model *m, double *grad_terms, double *grad_lik_sigma) {
  if (!m || !grad_terms) return fail(m ? m->ctx : nullptr, GPGP_EINVAL, "invalid argument");
  if (!m->fitted) return fail(m->ctx, GPGP_ENOT_FITTED, "model is not fitted");
  if (m->improper)
    return fail(m->ctx, GPGP_ENOT_FITTED, "the fit has no posterior (log_evidence = -Inf, improper bad-site posterior)");
  if (m->lik.kind != GPGP_LIK_GAUSSIAN || m->method.kind != GPGP_METHOD_FULL)
    return fail(m->ctx, GPGP_EUNSUPPORTED, "gradient needs lik_gaussian and method_full");
  gpgp_ctx *ctx = m->ctx;
  return guarded(ctx, [&]() -> gpgp_status {
    GPGP_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    const int64_t n = m->n;
    DBuf Bi, part, g, dg, red;
    compute_linv(m);
    Bi.alloc(s, (size_t)n * n);
    {
      // B^-1 = W^T W (lower part), W = L^-1
      Phase ph(ctx, GPGP_PHASE_LAUUM);
      if (m->opts.precision == GPGP_PREC_MIXED)
        lauum_mixed(s, m->Linv.p, n, n, Bi.p, n, m->errflag.p);
      else
        gemm64(s, true, false, n, n, n, 1.0, m->Linv.p, n, m->Linv.p, n, 0.0, Bi.p, n, true, 1);
    }
    // tr(C^-1) = sum_i s_i^2 Binv_ii
    dg.alloc(s, n);
    diag_scaled_kernel<<<g1(n), 256, 0, s>>>(n, Bi.p, m->s.p, dg.p);
    GPGP_CHECK_LAUNCH();
    red.alloc(s, 256);
    sum_vec(s, dg.p, n, red.p + 200);
    dot_partial(s, n, m->alpha.p, m->alpha.p, red.p);
    std::vector<double> hg(m->dk.nterms * GPGP_TERM_NPARAM);
    double h2[2];
    if (m->have_dK) {
      // the derivative matrices written with K: one pass over Binv and them, with
      // alpha alpha^T - diag(s) Binv diag(s) formed on the fly
      part.alloc(s, grad_stored_partials(n));
      g.alloc(s, GPGP_GRAD_MAXMAT + 1);
      {
        Phase ph(ctx, GPGP_PHASE_GRAD);
        grad_stored_contract(s, m->gplan, n, Bi.p, n, m->alpha.p, m->s.p, m->dK.p, n, (int64_t)n * n, part.p, g.p,
                             m->opts.precision == GPGP_PREC_MIXED);
      }
      double hs[GPGP_GRAD_MAXMAT + 1];
      GPGP_CUDA(cudaMemcpyAsync(hs, g.p, (m->gplan.m.nmat + 1) * sizeof(double), cudaMemcpyDeviceToHost, s));
      GPGP_CUDA(cudaMemcpyAsync(&h2[0], red.p + 200, sizeof(double), cudaMemcpyDeviceToHost, s));
      GPGP_CUDA(cudaMemcpyAsync(&h2[1], red.p + 64, sizeof(double), cudaMemcpyDeviceToHost, s));
      GPGP_CUDA(cudaStreamSynchronize(s));
      grad_stored_assemble(m->gplan, m->dk.nterms, hs, hg.data());
      m->dK.reset();  // made for this fit's gradient only
      m->have_dK = false;
    } else {
      dim3 gg((unsigned)std::min<int64_t>((n + 255) / 256, 64), (unsigned)std::min<int64_t>(n, 65535));
      grad_w_kernel<<<gg, 256, 0, s>>>(n, m->alpha.p, m->s.p, Bi.p);
      GPGP_CHECK_LAUNCH();
      part.alloc(s, cov_grad_partials(n));
      g.alloc(s, GPGP_MAX_TERMS * GPGP_TERM_NPARAM);
      gpgp_status st;
      {
        Phase ph(ctx, GPGP_PHASE_GRAD);
        st = cov_grad_contract(s, m->dk, m->F.p, n, n, Bi.p, n, part.p, g.p);
      }
      if (st != GPGP_OK) return fail(ctx, st, "gradient contraction failed");
      GPGP_CUDA(cudaMemcpyAsync(hg.data(), g.p, hg.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
      GPGP_CUDA(cudaMemcpyAsync(&h2[0], red.p + 200, sizeof(double), cudaMemcpyDeviceToHost, s));
      GPGP_CUDA(cudaMemcpyAsync(&h2[1], red.p + 64, sizeof(double), cudaMemcpyDeviceToHost, s));
      GPGP_CUDA(cudaStreamSynchronize(s));
    }
    if (tc_error(m)) return fail(ctx, GPGP_ETIMEOUT, "a tensor-core kernel wait timed out");
    for (size_t i = 0; i < hg.size(); ++i) grad_terms[i] = 0.5 * hg[i];
    if (grad_lik_sigma) {
      const double s2 = m->lik.sigma * m->lik.sigma;
      *grad_lik_sigma = s2 * (h2[1] - h2[0]);
    }
    return GPGP_OK;
  });
}

gpgp_status gpgp_cov_df_selftest(gpgp_ctx *ctx, const gpgp_kernel *k, const double *x, int64_t n, int32_t d,
                                 double jitter, double *max_rel_err) {
  if (!ctx || !k || !x || n < 1 || d < 1 || !max_rel_err) return fail(ctx, GPGP_EINVAL, "invalid argument");
  return guarded(ctx, [&]() -> gpgp_status {
    GPGP_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    DevKernel dk;
    std::vector<HostTermPrep> prep;
    std::string err;
    gpgp_status st = build_dev_kernel(k, d, &dk, &prep, &err);
    if (st != GPGP_OK) return fail(ctx, st, err);
    if (!cov_df_eligible(dk)) return fail(ctx, GPGP_EUNSUPPORTED, "kernel has no double-float path");
    GradPlan pl;
    if (!plan_grad_store(dk, &pl)) return fail(ctx, GPGP_EUNSUPPORTED, "too many derivative matrices");
    const int nm = pl.m.nmat;
    DBuf dx, F, K64, Kdf, D64, Ddf;
    copy_in(s, dx, x, (size_t)n * d, false);
    F.alloc(s, (size_t)n * std::max(1, dk.nfeat));
    prep_features(s, dk, prep, dx.p, n, n, F.p, n);
    K64.alloc(s, (size_t)n * n);
    Kdf.alloc(s, (size_t)n * n);
    D64.alloc(s, (size_t)std::max(1, nm) * n * n);
    Ddf.alloc(s, (size_t)std::max(1, nm) * n * n);
    GPGP_CUDA(cudaMemsetAsync(D64.p, 0, D64.n * sizeof(double), s));
    GPGP_CUDA(cudaMemsetAsync(Ddf.p, 0, Ddf.n * sizeof(double), s));
    cov_matrix_grad(s, dk, pl, F.p, n, n, K64.p, n, jitter, D64.p, n, (int64_t)n * n);
    IBuf derr;
    derr.alloc(s, 1);
    GPGP_CUDA(cudaMemsetAsync(derr.p, 0, sizeof(int), s));
    cov_matrix_df(s, dk, &pl, F.p, n, n, Kdf.p, n, jitter, Ddf.p, n, (int64_t)n * n, derr.p);
    std::vector<double> a((size_t)n * n), b((size_t)n * n);
    double out[2] = {0.0, 0.0};
    for (int q = -1; q < nm; ++q) {
      const double *pa = q < 0 ? K64.p : D64.p + (size_t)q * n * n;
      const double *pb = q < 0 ? Kdf.p : Ddf.p + (size_t)q * n * n;
      GPGP_CUDA(cudaMemcpyAsync(a.data(), pa, a.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
      GPGP_CUDA(cudaMemcpyAsync(b.data(), pb, b.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
      GPGP_CUDA(cudaStreamSynchronize(s));
      double mx = 0.0, dmax = 0.0;
      for (int64_t j = 0; j < n; ++j)
        for (int64_t i = j; i < n; ++i) mx = std::max(mx, std::fabs(a[i + j * n]));
      double rmax = 0.0;
      for (int64_t j = 0; j < n; ++j)
        for (int64_t i = j; i < n; ++i) {
          const double e = std::fabs(a[i + j * n] - b[i + j * n]);
          if (!(e == e)) return fail(ctx, GPGP_ENAN, "NaN in a covariance");
          dmax = std::max(dmax, e);
          if (std::fabs(a[i + j * n]) > 1e-20 * mx) rmax = std::max(rmax, e / std::fabs(a[i + j * n]));
        }
      out[0] = std::max(out[0], mx > 0.0 ? dmax / mx : dmax);
      if (q < 0) out[1] = rmax;
    }
    max_rel_err[0] = out[0];
    max_rel_err[1] = out[1];
    return GPGP_OK;
  });
}

}  // extern "C"
