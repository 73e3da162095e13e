// Context and model objects shared by the orchestration files (api.cu, fitc.cu).
#pragma once
#include <math.h>

#include <memory>
#include <new>
#include <string>
#include <utility>
#include <vector>

#include "common.cuh"

struct gpgp_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string last_error;
  double *h_pinned = nullptr;  // host pinned scalars
  // live profiling: (phase, start event, stop event) per recorded interval
  bool prof = false;
  bool prof_kernels = false;  // per-launch timers as well (single-stream Cholesky)
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> prof_ev;
  double prof_ms[GPGP_NPHASE] = {0};
  int64_t prof_calls[GPGP_NPHASE] = {0};
  gpgp::KernelTimer kt;
  gpgp::SideStream side;  // lookahead stream of the mixed Cholesky
};

namespace gpgp {

// Scoped phase timer: records a pair of events on the context stream when enabled.
struct Phase {
  gpgp_ctx *c;
  int ph;
  cudaEvent_t a = nullptr, b = nullptr;
  Phase(gpgp_ctx *ctx, int phase) : c(ctx), ph(phase) {
    if (!c->prof) return;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    cudaEventRecord(a, c->stream);
  }
  ~Phase() {
    if (!c->prof || !a) return;
    cudaEventRecord(b, c->stream);
    c->prof_ev.push_back({ph, {a, b}});
  }
};

inline void prof_collect(gpgp_ctx *c) {
  for (auto &e : c->prof_ev) {
    float ms = 0.f;
    cudaEventSynchronize(e.second.second);
    cudaEventElapsedTime(&ms, e.second.first, e.second.second);
    c->prof_ms[e.first] += ms;
    c->prof_calls[e.first] += 1;
    cudaEventDestroy(e.second.first);
    cudaEventDestroy(e.second.second);
  }
  c->prof_ev.clear();
}

// RAII device buffer on the context's stream-ordered pool.
struct DBuf {
  double *p = nullptr;
  size_t n = 0;
  cudaStream_t s = nullptr;
  DBuf() = default;
  DBuf(const DBuf &) = delete;
  DBuf &operator=(const DBuf &) = delete;
  ~DBuf() { reset(); }
  void alloc(cudaStream_t st, size_t count) {
    reset();
    s = st;
    n = count;
    if (count == 0) return;
    cudaError_t e = cudaMallocAsync((void **)&p, count * sizeof(double), st);
    if (e != cudaSuccess) {
      p = nullptr;
      (void)cudaGetLastError();
      throw std::bad_alloc();
    }
  }
  void reset() {
    if (p) cudaFreeAsync(p, s);
    p = nullptr;
    n = 0;
  }
};

struct IBuf {
  int *p = nullptr;
  cudaStream_t s = nullptr;
  IBuf() = default;
  IBuf(const IBuf &) = delete;
  IBuf &operator=(const IBuf &) = delete;
  ~IBuf() {
    if (p) cudaFreeAsync(p, s);
  }
  void alloc(cudaStream_t st, size_t count) {
    if (p) cudaFreeAsync(p, s);
    s = st;
    if (cudaMallocAsync((void **)&p, count * sizeof(int), st) != cudaSuccess) {
      p = nullptr;
      (void)cudaGetLastError();
      throw std::bad_alloc();
    }
  }
};

// Resident quantities of a FITC fit (R/gp_fit.R:101-123, R/linear_algebra.R:3-43).
struct FitcState {
  int64_t M = 0;
  DBuf z, Fz;           // inducing inputs (M x d) and their features
  DBuf Kz, Lz, Wz_blk;  // K(z,z) + jitter I, its factor, diagonal-block inverses
  DBuf Kxz;             // K(x, z), n x M
  DBuf X;               // Kxz Lz^-T = t(forwardsolve(Kz_chol, t(Kxz))), n x M
  DBuf D, Kdiag;        // FITC diagonal (with jitter) and diag K(x, x)
  DBuf S, iDU;          // S = D + V, inv_D_U = Kxz / S (n x M)
  DBuf Cm, Lm, Wm_blk;  // K_z + U^T S^-1 U and its factor
  double logdet = 0.0;  // log det of the lemma's matrix (R/linear_algebra.R:30-34)
  // prediction caches (independent of the test points), filled on first use:
  // Sig1 holds sol = A1 S^-1 A1^T - P C_m^-1 P^T, P = A1 inv_D_U
  DBuf Sig1, P;
  bool have_pred_cache = false;
};

// Blocks of a method_full fit whose last iteration took the non-log-concave
// branch (nlc.cu): the good sites' factor and the Schur complement of the bad
// ones, in place of a factor of B over all sites.
struct NlcState {
  int64_t ng = 0, nb = 0;
  IBuf good, bad;       // site indices (V > 0, V <= 0)
  DBuf sg, L1, W1;      // 1/sqrt(V_good), lower factor of B_good, its diagonal-block inverses
  DBuf aux;             // L1^-1 s_good K(good, bad), ng x nb
  DBuf Slu;             // LU of S = pred_cov + diag(V_bad), nb x nb
  IBuf piv;
  DBuf Fg, Fb;          // features of the good / bad training rows, filled on first prediction
};

// One term of a random-feature map (rf.cu).
enum RfKind { RF_CONST = 0, RF_LIN = 1, RF_SEXP = 2, RF_NN = 3, RBF_SEXP = 4 };
struct RfTerm {
  int kind;      // RfKind
  int group;     // the cf (group) whose features this term multiplies into
  int off;       // first input column of the term in the feature matrix F
  int q;         // input columns of the term
  int nb;        // features of the group
  int64_t doff;  // offset of the term's draws in the packed draws array
  double magn, lscale, sigma0, sigma;
};
struct RfSpec {
  int nterms = 0, ngroups = 0, D = 0;
  int gcol0[GPGP_MAX_TERMS + 1];  // first column of each group in the feature matrix; [ngroups] = D
  RfTerm t[GPGP_MAX_TERMS];
};
// Host side: the feature map of (kernel, method) from the method's draws; packs
// the draws into *draws. Errors as the reference's feature-map constructors.
gpgp_status build_rf_spec(const gpgp_kernel *k, const gpgp_method *me, const DevKernel &dk, RfSpec *sp,
                          std::vector<double> *draws, std::string *err);

// Resident quantities of a method_rf / method_rbf fit (R/laplace.R:241-262).
struct RfState {
  RfSpec spec;
  DBuf dr;               // packed draws
  DBuf Z;                // features of the training inputs, n x D
  DBuf L, Wblk;          // factor of Z^T diag(1/V) Z + I and its diagonal-block inverses
  DBuf W;                // L^-1 (strict upper zero)
  DBuf wmean, wcov;      // weight posterior
};

}  // namespace gpgp

struct gpgp_model {
  gpgp_ctx *ctx = nullptr;
  gpgp_kernel spec;
  gpgp::DevKernel dk;
  std::vector<gpgp::HostTermPrep> prep;
  gpgp_lik lik;
  gpgp::LikDev lk;
  gpgp_method method;
  gpgp_approx approx;
  gpgp_fit_opts opts;
  int64_t n = 0;
  int d = 0;
  // inputs (owned copies)
  gpgp::DBuf x, y, trials, offset, F;
  // full-method fit
  gpgp::DBuf L, Winv, s, alpha, fmean, z, V;
  gpgp::DBuf fvar, cav_mean, cav_var;  // EP
  gpgp::DBuf binv_diag;                // diag(B^-1), filled on demand
  bool have_binv_diag = false;
  gpgp::DBuf Linv;                     // W = L^-1, kept resident once computed
  bool have_Linv = false;
  bool want_linv = false;              // the gradient follows the fit: form L^-1 right after the factor (mixed)
  bool want_dk = false;                // the gradient follows the fit: write K's derivative matrices with K
  gpgp::DBuf dK;                       // those matrices (plan gplan), valid while have_dK
  gpgp::GradPlan gplan;
  bool have_dK = false;
  bool b_ready = false;                // B = I + K / sigma^2 already written into L by the covariance kernel
  gpgp::IBuf errflag;                  // bounded-wait timeouts of the device kernels
  std::unique_ptr<gpgp::FitcState> fitc;
  std::unique_ptr<gpgp::NlcState> nlc;  // set when the last iteration was non-log-concave
  std::unique_ptr<gpgp::RfState> rf;    // method_rf / method_rbf
  bool improper = false;  // the reference's -Inf fit without a posterior (chol(A) failed)
  bool has_trials = false, has_offset = false;
  double log_evidence = 0.0;
  int fitted = 0;
  int64_t fp64_fallbacks = 0;  // mixed factorisations redone in FP64 after a breakdown
};

namespace gpgp {

extern thread_local std::string tl_error;

inline gpgp_status fail(gpgp_ctx *ctx, gpgp_status st, const std::string &msg) {
  if (ctx) ctx->last_error = msg;
  tl_error = msg;
  return st;
}

// binds the context's kernel timer to this thread for one API call
struct KTBind {
  KernelTimer *prev;
  explicit KTBind(gpgp_ctx *ctx) : prev(tl_kt) { tl_kt = (ctx && ctx->prof && ctx->prof_kernels) ? &ctx->kt : nullptr; }
  ~KTBind() { tl_kt = prev; }
};

template <class F>
gpgp_status guarded(gpgp_ctx *ctx, F &&fn) {
  KTBind bind(ctx);
  try {
    return fn();
  } catch (const CudaError &e) {
    (void)cudaGetLastError();  // a launch error is not sticky: do not leave it pending
    std::string m = std::string("CUDA error ") + cudaGetErrorString(e.err) + " in " + e.what;
    return fail(ctx, GPGP_ECUDA, m);
  } catch (const std::bad_alloc &) {
    return fail(ctx, GPGP_EOOM, "device or host allocation failed");
  }
}

inline LikDev make_likdev(const gpgp_lik &l) {
  LikDev d;
  d.kind = l.kind;
  d.link = l.link;
  d.sigma = l.sigma;
  d.phi = l.phi;
  return d;
}

inline void copy_in(cudaStream_t s, DBuf &dst, const double *src, size_t count, bool src_on_device) {
  dst.alloc(s, count);
  if (count == 0) return;
  GPGP_CUDA(cudaMemcpyAsync(dst.p, src, count * sizeof(double),
                            src_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s));
}

inline double read_scalar(gpgp_ctx *ctx, const double *dptr) {
  GPGP_CUDA(cudaMemcpyAsync(ctx->h_pinned, dptr, sizeof(double), cudaMemcpyDeviceToHost,
                            ctx->stream));
  GPGP_CUDA(cudaStreamSynchronize(ctx->stream));
  return ctx->h_pinned[0];
}

inline unsigned g1(int64_t n) { return (unsigned)((n + 255) / 256 > 0 ? (n + 255) / 256 : 1); }

// FITC orchestration (fitc.cu)
gpgp_status fit_fitc(gpgp_model *m, gpgp_fit_result *res, const double *inducing, bool on_device);
gpgp_status pred_fitc(gpgp_model *m, const double *Ft, int64_t mt, uint32_t gm, double *mean,
                      double *var);
gpgp_status loo_fitc_posteriors(gpgp_model *m, double *lmean, double *lvar);
gpgp_status pred_cov_fitc(gpgp_model *m, const double *Ft, int64_t mt, uint32_t gm, double jitter, double *mean,
                          double *C);

// method_rf / method_rbf (rf.cu): fit, predictive mean / variance at test features
// Ft (mt rows), posterior variances at the training inputs (LOO).
gpgp_status fit_rf(gpgp_model *m, gpgp_fit_result *res);
gpgp_status pred_rf(gpgp_model *m, const double *Ft, int64_t mt, uint32_t gm, double *mean, double *var);
void rf_train_var(gpgp_model *m, double *var);

// Non-log-concave branch of a method_full Laplace / EP iteration (nlc.cu).
gpgp_status nlc_fit_full(gpgp_model *m, const double *K, const double *logC, bool ep, double *alpha, double *fnew,
                         double *fvar, double *lml, bool *improper);
// Predictive variances (device, mt) of a fit in m->nlc at test features Ft (mt rows).
void nlc_pred_var(gpgp_model *m, const double *Ft, int64_t mt, uint32_t gm, double *var);
// The bad sites' terms of the split given their prior N(pm, pc) (nlc.cu).
gpgp_status nlc_bad_terms(gpgp_model *m, int64_t nb, const int *bad, const double *pm, const double *pc,
                          const double *zb, const double *Vb, const double *yb, const double *tb, const double *ob,
                          bool ep, const double *logC, double *lml2, double *lpu2, bool *improper);
void gather_rows(cudaStream_t s, const double *F, int64_t ldf, int64_t nf, const int *idx, int64_t m, double *out);
void split_sites(gpgp_model *m, std::vector<int> *hg, std::vector<int> *hb, IBuf *good, IBuf *bad);

// Batched pipeline for the request server (batched.cu): one plan, one run, no
// autotune or graph; lml[nprob], mean/var[sum m] packed in problem order.
gpgp_status batch_solve_once(gpgp_ctx *ctx, const gpgp_batch_problem *probs, int32_t nprob,
                             int32_t precision, double jitter, double *lml, double *mean, double *var);
size_t batch_bytes_estimate(int64_t n, int64_t m, int32_t d, int32_t precision);

}  // namespace gpgp
