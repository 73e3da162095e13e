/*
 * gpgp.h -- C ABI of the GB300 Gaussian-process library (libgpgp.so).
 *
 * This is the drop-in boundary for gplite's GP hot path. The R package
 * gplite binds exactly four native routines today (src/RcppExports.cpp:76-87:
 * _gplite_cf_sexp_c, _gplite_cf_matern32_c, _gplite_cf_matern52_c,
 * _gplite_cf_nn_c); everything else is R calling LAPACK. The functions below
 * keep those four covariance routines (gpgp_cf_*) and add whole-fit entry
 * points that replace the S3 seams fit_model / gp_pred_post / loo_posteriors
 * (R/gp_fit.R:62-188, R/gp_pred.R:129-296, R/gp_loo.R:111-133), so that the
 * covariance, Cholesky, solves and evidence never leave the GPU.
 *
 * Conventions
 *  - Matrices are column-major double, like R matrices: x is n-by-d with
 *    element (i, k) at x[i + k*n].
 *  - Host-pointer entry points copy inputs in and results out; *_dev entry
 *    points take device pointers that stay owned by the caller.
 *  - The library owns device memory of contexts and models. A context is
 *    bound to one device and one stream and is not thread-safe; use one
 *    context per host thread.
 *  - Every call returns a gpgp_status; no call aborts or traps. Numerical
 *    failures the reference maps to log_evidence = -Inf (non-PD factor,
 *    NaN sites, EP max-iterations) are reported in gpgp_fit_result and the
 *    log_evidence field, exactly where the reference does.
 */
#ifndef GPGP_H
#define GPGP_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GPGP_MAX_VARS 16
#define GPGP_MAX_TERMS 16
#define GPGP_TERM_NPARAM 5 /* lscale, magn, sigma0, sigma, period */

typedef enum gpgp_status {
  GPGP_OK = 0,
  GPGP_ENOT_PD = 1,       /* Cholesky met a non-positive pivot (see result.info) */
  GPGP_ENAN = 2,          /* NaN/Inf in inputs or in site parameters */
  GPGP_EMAXITER = 3,      /* iteration limit reached (Laplace / EP) */
  GPGP_EUNSUPPORTED = 4,  /* combination not available (e.g. EP with method_rf, as in the reference) */
  GPGP_EOOM = 5,          /* device allocation failed or budget exceeded */
  GPGP_ETIMEOUT = 6,      /* a bounded device wait ran out */
  GPGP_ECUDA = 7,         /* CUDA runtime error (message in gpgp_last_error) */
  GPGP_EINVAL = 8,        /* invalid argument */
  GPGP_ENOT_FITTED = 9,   /* model handle has no fit */
  GPGP_EBUSY = 10         /* server queue full / request not finished */
} gpgp_status;

/* Covariance function kinds (R/cf.R:92-195, src/cf.cpp). cf_periodic is a
 * flag on a term (inputs mapped to sin/cos of 2*pi*x/period, R/cf.R:478-489)
 * whose kind is that of its base kernel; cf_prod is expressed with groups. */
typedef enum gpgp_cf_kind {
  GPGP_CF_CONST = 0,
  GPGP_CF_LIN = 1,
  GPGP_CF_SEXP = 2,
  GPGP_CF_MATERN32 = 3,
  GPGP_CF_MATERN52 = 4,
  GPGP_CF_NN = 5
} gpgp_cf_kind;

/* One covariance term. Terms with the same group id are multiplied
 * (eval_cf.cf_prod, R/cf.R:491-497); groups are summed (eval_cf.list,
 * R/cf.R:402-411). Group ids are 0..ngroups-1 and terms of one group are
 * contiguous. Parameter values are natural (not log). */
typedef struct gpgp_cf_term {
  int32_t kind;      /* gpgp_cf_kind (of the base kernel when periodic) */
  int32_t group;     /* product group == index of the cf in the gp's cfs list */
  int32_t periodic;  /* 1: cf_periodic wrapping this base kernel */
  int32_t normalize; /* 1: (x - means) / scales before use (R/misc.R:17-31) */
  int32_t nvars;     /* number of input columns used; 0 = all d columns */
  int32_t vars[GPGP_MAX_VARS];     /* 0-based column indices */
  double means[GPGP_MAX_VARS];     /* learn_scales output (R/cf.R:836-845) */
  double scales[GPGP_MAX_VARS];
  double lscale, magn, sigma0, sigma, period;
} gpgp_cf_term;

typedef struct gpgp_kernel {
  int32_t nterms;
  int32_t ngroups;
  gpgp_cf_term term[GPGP_MAX_TERMS];
} gpgp_kernel;

typedef enum gpgp_lik_kind {
  GPGP_LIK_GAUSSIAN = 0,
  GPGP_LIK_BERNOULLI = 1,
  GPGP_LIK_BINOMIAL = 2,
  GPGP_LIK_POISSON = 3,
  GPGP_LIK_BETABINOM = 4
} gpgp_lik_kind;

typedef enum gpgp_link {
  GPGP_LINK_IDENTITY = 0,
  GPGP_LINK_LOGIT = 1,
  GPGP_LINK_PROBIT = 2,
  GPGP_LINK_LOG = 3
} gpgp_link;

/* Likelihood (R/lik.R:44-90). */
typedef struct gpgp_lik {
  int32_t kind;
  int32_t link;
  double sigma; /* lik_gaussian noise sd */
  double phi;   /* lik_betabinom over-dispersion */
} gpgp_lik;

typedef enum gpgp_method_kind {
  GPGP_METHOD_FULL = 0,
  GPGP_METHOD_FITC = 1,
  GPGP_METHOD_RF = 2, /* random features (R/method.R:129-133) */
  GPGP_METHOD_RBF = 3 /* radial basis features at training inputs (R/method.R:135-139) */
} gpgp_method_kind;

/* Method (R/method.R:105-139). For FITC the inducing inputs are given
 * explicitly (M-by-d column-major, host memory for gpgp_fit, device memory
 * for gpgp_fit_dev).
 * For method_rf / method_rbf the random draws of the reference's feature maps
 * (rf_featmap / rbf_featmap, R/cf.R:532-817) are given explicitly, in host
 * memory, per term (terms as in gpgp_kernel), with q the term's input count
 * (nvars, or 2 nvars for cf_periodic) and nb = num_basis of its group:
 *   rf, cf_sexp: q x nb/2 standard normals (column-major; R's `w` before the
 *                scaling by 1/lscale), features [cos(h), sin(h)], h = x w;
 *   rf, cf_nn:   q x nb standard normals, then nb more (R's `w` and `w0`
 *                before their scaling by sigma and sigma0 sigma);
 *   rbf, cf_sexp: q x nb centres (column j = centre j, in the term's input
 *                space: the raw training inputs of its columns, or their
 *                sin/cos transform under cf_periodic);
 *   cf_const, cf_lin: none (NULL); their groups take 1 and nvars features.
 * cf_matern32/52 have no feature map (an error in the reference too). */
typedef struct gpgp_method {
  int32_t kind;
  int32_t num_inducing;
  const double *inducing;
  int32_t num_basis[GPGP_MAX_TERMS];    /* features per group (rf / rbf) */
  const double *draws[GPGP_MAX_TERMS];  /* per term (rf / rbf), see above */
} gpgp_method;

typedef enum gpgp_approx_kind { GPGP_APPROX_LAPLACE = 0, GPGP_APPROX_EP = 1 } gpgp_approx_kind;

/* Latent approximation (R/approx.R:60-75); EP also uses damping_min and tol
 * (R/gp_fit.R:150-161: damping_min 0.1, tol 1e-4 full / 1e-3 FITC). */
typedef struct gpgp_approx {
  int32_t kind;
  int32_t maxiter;
  double tol;
  double damping;
  double damping_min;
  int32_t quad_order;
} gpgp_approx;

typedef enum gpgp_precision {
  GPGP_PREC_FP64 = 0,  /* plain: FP64 throughout */
  GPGP_PREC_MIXED = 1  /* BF16-split tensor-core updates, FP64 diagonal blocks,
                          FP64 log-determinant and FP64 iterative refinement */
} gpgp_precision;

typedef struct gpgp_fit_opts {
  double jitter;        /* diagonal jitter (R/gp.R:276-281 default 1e-6) */
  int32_t precision;    /* gpgp_precision */
  int32_t refine_iters; /* FP64 iterative-refinement steps for alpha (mixed) */
} gpgp_fit_opts;

typedef struct gpgp_fit_result {
  double log_evidence; /* -Inf where the reference returns -Inf */
  int32_t status;      /* gpgp_status of the numerical outcome */
  int32_t iters;       /* Laplace / EP iterations used */
  int64_t info;        /* first non-PD pivot (1-based) when status == GPGP_ENOT_PD */
  int32_t quad_ok;     /* EP quadrature produced no NaN (R/lik.R:250-257) */
  int32_t converged;   /* 0 if the iteration limit was reached */
  int32_t precision_used; /* GPGP_PREC_FP64 when a mixed Laplace / EP fit broke down
                             (pseudo-variance <= 0, NaN) and was redone in FP64 */
} gpgp_fit_result;

typedef struct gpgp_ctx gpgp_ctx;
typedef struct gpgp_model gpgp_model;

/* ---- context ---------------------------------------------------------- */
/* A context owns a CUDA stream (all its work is ordered on it) and two side
   streams that the mixed-precision Cholesky uses for its lookahead; calls on one
   context must not overlap, separate contexts may run from separate threads.
   Device memory comes from the device's default stream-ordered pool; creating a
   context raises that pool's release threshold to a quarter of the device's
   memory (when it is lower), so that memory freed at the end of a fit is reused
   by the next one instead of being unmapped at every synchronisation and mapped
   again. The setting belongs to this process and ends with it. */
gpgp_status gpgp_create(gpgp_ctx **ctx, int device);
gpgp_status gpgp_destroy(gpgp_ctx *ctx);
const char *gpgp_status_string(gpgp_status s);
const char *gpgp_last_error(const gpgp_ctx *ctx);
/* Kernel launches issued by this context since creation (evidence counter). */
int64_t gpgp_launch_count(const gpgp_ctx *ctx);
/* Synchronise the context's stream. */
gpgp_status gpgp_sync(gpgp_ctx *ctx);
/* The context's cudaStream_t, as an opaque pointer. */
void *gpgp_stream(gpgp_ctx *ctx);

/* ---- live profiling: CUDA events recorded on the context's stream around
 *      each phase of the hot path; read back as total milliseconds and
 *      call counts per phase. Enabling resets the accumulators. on = 1 also
 *      times every dense-contraction launch alone (below), which makes the
 *      mixed Cholesky run on one stream; on = 2 times the phases only and
 *      keeps the lookahead schedule. on = 0 stops profiling. -------------- */
typedef enum gpgp_phase {
  GPGP_PHASE_COV = 0,      /* covariance matrix generation */
  GPGP_PHASE_POTRF = 1,    /* blocked Cholesky */
  GPGP_PHASE_SOLVE = 2,    /* triangular solves for alpha, K alpha */
  GPGP_PHASE_TRTRI = 3,    /* triangular inverse */
  GPGP_PHASE_LAUUM = 4,    /* B^-1 = L^-T L^-1 */
  GPGP_PHASE_GRAD = 5,     /* gradient contraction */
  GPGP_PHASE_PRED_MEAN = 6,
  GPGP_PHASE_PRED_VAR = 7, /* cross covariance + multi-RHS solve */
  GPGP_NPHASE = 8
} gpgp_phase;
gpgp_status gpgp_profile_enable(gpgp_ctx *ctx, int32_t on);
gpgp_status gpgp_profile_read(gpgp_ctx *ctx, double *ms, int64_t *calls);
/* Per-kernel timing of the dense contractions (instrumentation, no
 * counterpart in the reference): while profiling is on, each launch of these
 * kernels made through this context is bracketed by CUDA events on the
 * context stream. Read per kernel: launches, total device ms, and the
 * arithmetic the launches executed (tensor-core GEMM: BF16 MMA flops of all
 * slice products of the tiles it ran; FP64 GEMM: 2 x tile area x K of the
 * tiles it ran). Reset by gpgp_profile_enable. */
typedef enum gpgp_kprof_kernel {
  GPGP_KPROF_OZ_GEMM = 0,     /* BF16-sliced tcgen05 GEMM (mixed precision) */
  GPGP_KPROF_GEMM64 = 1,      /* FP64 GEMM / SYRK (plain precision) */
  GPGP_KPROF_POTRF_DIAG = 2,  /* 64 x 64 diagonal-block factor + inverse (flops: 2 x 64^3 / 3) */
  GPGP_KPROF_OZ_SPLIT = 3,    /* FP64 -> BF16 slices (flops: 0; elements split) */
  GPGP_KPROF_TRSV = 4,        /* cooperative triangular solve (flops: n^2) */
  GPGP_NKPROF = 5
} gpgp_kprof_kernel;
gpgp_status gpgp_kernel_profile_read(gpgp_ctx *ctx, int32_t kernel, int64_t *launches, double *ms,
                                     double *flops);

/* ---- covariance routines: replace src/cf.cpp:9-162 (registered at
 *      src/RcppExports.cpp:76-87). Host buffers; x1 n1-by-d, x2 n2-by-d
 *      column-major; out n1-by-n2 column-major, or min(n1,n2) if diag_only.
 *      They run on an internal context for device 0. ---------------------- */
gpgp_status gpgp_cf_sexp(const double *x1, int64_t n1, const double *x2, int64_t n2, int32_t d,
                         double lscale, double magn, int32_t diag_only, double *out);
gpgp_status gpgp_cf_matern32(const double *x1, int64_t n1, const double *x2, int64_t n2,
                             int32_t d, double lscale, double magn, int32_t diag_only,
                             double *out);
gpgp_status gpgp_cf_matern52(const double *x1, int64_t n1, const double *x2, int64_t n2,
                             int32_t d, double lscale, double magn, int32_t diag_only,
                             double *out);
gpgp_status gpgp_cf_nn(const double *x1, int64_t n1, const double *x2, int64_t n2, int32_t d,
                       double sigma0, double sigma, double magn, int32_t diag_only, double *out);

/* eval_cf.list (R/cf.R:402-411) for a whole kernel; group_mask selects the
 * cfs (bit g = group g; 0 = all), like the cfind argument. Host buffers. */
gpgp_status gpgp_eval_cf(gpgp_ctx *ctx, const gpgp_kernel *k, const double *x1, int64_t n1,
                         const double *x2, int64_t n2, int32_t d, int32_t diag_only,
                         uint32_t group_mask, double *out);

/* ---- fit: replaces gp_fit -> fit_model (R/gp_fit.R:54-188) ------------- */
/* Host buffers: x n-by-d, y n, trials n or NULL, offset n or NULL. The model
 * keeps x, y, the factor and the site parameters resident on the device. */
gpgp_status gpgp_fit(gpgp_ctx *ctx, const gpgp_kernel *k, const gpgp_lik *lik,
                     const gpgp_method *method, const gpgp_approx *approx,
                     const gpgp_fit_opts *opts, const double *x, int64_t n, int32_t d,
                     const double *y, const double *trials, const double *offset,
                     gpgp_model **model, gpgp_fit_result *result);
/* Same, with x, y, trials, offset (and method->inducing) in device memory. */
gpgp_status gpgp_fit_dev(gpgp_ctx *ctx, const gpgp_kernel *k, const gpgp_lik *lik,
                         const gpgp_method *method, const gpgp_approx *approx,
                         const gpgp_fit_opts *opts, const double *x, int64_t n, int32_t d,
                         const double *y, const double *trials, const double *offset,
                         gpgp_model **model, gpgp_fit_result *result);
gpgp_status gpgp_model_free(gpgp_model *model);

/* Gradient of log_evidence with respect to the log of every term parameter
 * (GPGP_TERM_NPARAM slots per term, order lscale, magn, sigma0, sigma,
 * period; unused slots are 0) and of log lik->sigma. Gaussian likelihood,
 * full method. This is tr((alpha alpha^T - C^-1) dC/dtheta)/2; the reference
 * has no gradient (it optimises with Nelder-Mead, R/gp_optim.R:94). */
gpgp_status gpgp_model_grad(gpgp_model *model, double *grad_terms, double *grad_lik_sigma);
/* gpgp_fit (gpgp_fit_dev) followed by gpgp_model_grad, in one call: the step of
 * a gradient-based gp_optim. Same arguments and outputs as the two calls (the
 * model is returned fitted). Knowing that the gradient follows, a mixed-precision
 * fit forms the triangular inverse L^-1 the gradient needs right after the
 * factorisation and solves for alpha with it (two matrix-vector products per
 * solve) instead of with the blocked triangular solves. lik_gaussian and
 * method_full only (GPGP_EUNSUPPORTED otherwise, as gpgp_model_grad). */
gpgp_status gpgp_fit_grad(gpgp_ctx *ctx, const gpgp_kernel *k, const gpgp_lik *lik, const gpgp_method *method,
                          const gpgp_approx *approx, const gpgp_fit_opts *opts, const double *x, int64_t n,
                          int32_t d, const double *y, const double *trials, const double *offset,
                          gpgp_model **model, gpgp_fit_result *result, double *grad_terms,
                          double *grad_lik_sigma);
gpgp_status gpgp_fit_grad_dev(gpgp_ctx *ctx, const gpgp_kernel *k, const gpgp_lik *lik, const gpgp_method *method,
                              const gpgp_approx *approx, const gpgp_fit_opts *opts, const double *x, int64_t n,
                              int32_t d, const double *y, const double *trials, const double *offset,
                              gpgp_model **model, gpgp_fit_result *result, double *grad_terms,
                              double *grad_lik_sigma);

/* Copy a resident model vector out to host memory (length n unless noted). */
typedef enum gpgp_model_field {
  GPGP_FIELD_ALPHA = 0,
  GPGP_FIELD_FMEAN = 1,
  GPGP_FIELD_Z = 2,
  GPGP_FIELD_V = 3,
  GPGP_FIELD_FVAR = 4,        /* EP posterior marginal variances */
  GPGP_FIELD_CAVITY_MEAN = 5, /* EP */
  GPGP_FIELD_CAVITY_VAR = 6,  /* EP */
  GPGP_FIELD_WMEAN = 7,       /* rf / rbf: posterior mean of the weights (D = sum of num_basis) */
  GPGP_FIELD_WCOV = 8         /* rf / rbf: posterior covariance of the weights (D x D) */
} gpgp_model_field;
gpgp_status gpgp_model_get(gpgp_model *model, int32_t field, double *out);

/* ---- prediction: replaces gp_pred_post.method_full / method_fitc
 *      (R/gp_pred.R:202-296). xt m-by-d; mean m; var m or NULL. ---------- */
gpgp_status gpgp_pred(gpgp_model *model, const double *xt, int64_t m, uint32_t group_mask,
                      double *mean, double *var);
gpgp_status gpgp_pred_dev(gpgp_model *model, const double *xt, int64_t m, uint32_t group_mask,
                          double *mean, double *var);

/* ---- full predictive covariance: gp_pred_post(cov = TRUE).method_full
 *      (R/gp_pred.R:202-232): mean (m) and cov (m x m, column-major)
 *      = K(xt, xt) - aux^T aux + jitter I, aux = C_chol^-1 K(x, xt). FP64.
 *      method_fitc returns GPGP_EUNSUPPORTED. ---- */
gpgp_status gpgp_pred_cov(gpgp_model *model, const double *xt, int64_t m, uint32_t group_mask,
                          double jitter, double *mean, double *cov);

/* ---- multivariate normal draws: mvnrnd (R/gp_draw.R:182-199),
 *      out = mean 1^T + t(chol(cov)) z for a caller-drawn standard-normal
 *      z (d x draws, column-major); FP64 Cholesky on the device. A
 *      covariance that is not positive definite gives GPGP_ENOT_PD (an error
 *      of R's chol in the reference). ---- */
gpgp_status gpgp_mvn_draw(gpgp_ctx *ctx, const double *mean, const double *cov, int64_t d,
                          const double *z, int64_t draws, double *out);

/* ---- random-feature methods without a fit: gp_pred_prior.method_rf
 *      (R/gp_pred.R:186-200) and gp_draw_prior.method_rf (R/gp_draw.R:87-103).
 *      The features zt (m x D_sel, the selected groups' columns) of xt
 *      (m x d, host memory) are formed on the device from method's draws;
 *      var (m, or NULL) = diag(zt zt^T); sample (m x draws, or NULL when
 *      z is NULL) = zt z for caller-drawn standard normals z (D_sel x draws,
 *      column-major). gpgp_pred / gpgp_loo / gpgp_model_get serve fitted
 *      rf / rbf models; gpgp_model_grad and gpgp_pred_cov return
 *      GPGP_EUNSUPPORTED for them, as the reference has neither. ---------- */
gpgp_status gpgp_rf_prior(gpgp_ctx *ctx, const gpgp_kernel *k, const gpgp_method *method,
                          const double *xt, int64_t m, int32_t d, uint32_t group_mask, double *var,
                          const double *z, int64_t draws, double *sample);
/* ---- posterior draws of a fitted rf / rbf model in weight space:
 *      gp_draw_analytic.method_rf (R/gp_draw.R:145-169),
 *      sample = zt (wmean + t(chol(wcov)) z) over the selected groups, z
 *      D_sel x draws standard normals (host, column-major), sample m x draws. */
gpgp_status gpgp_rf_draw(gpgp_model *model, const double *xt, int64_t m, uint32_t group_mask,
                         const double *z, int64_t draws, double *sample);

/* ---- k-means of the inducing inputs: stats::kmeans in get_inducing
 *      (R/gp_fit.R:192-236). Lloyd's algorithm from the caller's initial
 *      centres (k x d), at most max_iter iterations; deterministic centre
 *      sums. x n x d column-major, d <= 16, k d <= 6144. Writes the centres
 *      (k x d), the iterations used and the within-cluster sum of squares. */
gpgp_status gpgp_kmeans(gpgp_ctx *ctx, const double *x, int64_t n, int32_t d, int32_t k,
                        const double *init, int32_t max_iter, double *centers, int32_t *iters,
                        double *wss);

/* ---- LOO: replaces loo_posteriors + the quadrature of gp_loo
 *      (R/gp_loo.R:73-133) on the model's own training data. ------------- */
gpgp_status gpgp_loo(gpgp_model *model, int32_t quad_order, double *loos, double *loo_sum);
/* Monte Carlo LOO (gp_loo with quadrature = FALSE, R/gp_loo.R:97-103): z holds
 * n x draws standard normals (column-major, host memory; the reference draws them
 * with stats::rnorm in the same order), fsample = loo_mean + sqrt(loo_var) z and
 * loos_i = logsumexp_k log p(y_i | fsample_ik) - log(draws). */
gpgp_status gpgp_loo_mc(gpgp_model *model, int64_t draws, const double *z, double *loos,
                        double *loo_sum);

/* ---- batched small GPs: many independent regressions of uneven size --
 * Each problem is gp_fit (lik_gaussian, method_full, one covariance term of
 * kind sexp / matern32 / matern52 over all d inputs), gp_loo (approx_laplace,
 * Gauss-Hermite of order quad_order) and gp_pred with var = TRUE at its m test
 * points. Host buffers, column-major; n <= 4096, d <= 8. A plan uploads the
 * inputs, autotunes each size bucket (mixed precision: FP64 pipe or sliced
 * tensor cores, whichever is faster) and captures the whole pipeline in one
 * CUDA graph; gpgp_batch_run replays it; gpgp_batch_upload replaces the inputs
 * of a plan with new data of the same shapes. Results are packed in problem
 * order: log_evidence[nprob], mean/var[sum m_i], loos[sum n_i]. A problem whose
 * factor is not positive definite gets log_evidence = -Inf. */
typedef struct gpgp_batch_problem {
  int32_t n, d, m;
  int32_t kind;                /* GPGP_CF_SEXP, GPGP_CF_MATERN32 or GPGP_CF_MATERN52 */
  double lscale, magn, sigma;  /* cf lscale, cf magn, lik_gaussian sigma */
  const double *x, *y, *xt;
} gpgp_batch_problem;
typedef struct gpgp_batch gpgp_batch;
gpgp_status gpgp_batch_create(gpgp_ctx *ctx, const gpgp_batch_problem *probs, int32_t nprob,
                              int32_t precision, int32_t quad_order, double jitter,
                              gpgp_batch **out);
gpgp_status gpgp_batch_upload(gpgp_batch *b, const gpgp_batch_problem *probs);
gpgp_status gpgp_batch_run(gpgp_batch *b);
gpgp_status gpgp_batch_results(gpgp_batch *b, double *log_evidence, double *mean, double *var,
                               double *loos);
gpgp_status gpgp_batch_info(gpgp_batch *b, int32_t *nbuckets, int32_t *bucket_n,
                            int32_t *bucket_count, int32_t *bucket_variant, double *tune_ms);
gpgp_status gpgp_batch_destroy(gpgp_batch *b);

/* ---- request server: continuous batching of fit + predict requests -----
 * Serves gp_fit (+ gp_pred with var) and gp_pred-on-a-resident-model requests
 * that arrive one by one (the reference has no counterpart: it is one R call
 * per fit). gpgp_server_submit copies the request's inputs and returns at
 * once. Requests are admitted in arrival order while their device memory
 * estimate fits the HBM budget (a later, smaller request may pass one that
 * does not fit, until that one has waited 100 ms); a request larger than the
 * whole budget fails with GPGP_EOOM. Admitted Gaussian full-method requests
 * with one sexp / matern32 / matern52 term over all inputs and n <= batch_max_n
 * join the batch lane: whatever has gathered while the previous batch ran is
 * solved as the next batch (the batched pipeline, one launch sequence for all);
 * the others (Laplace / EP likelihoods, FITC, compound kernels, large n) run on
 * a pool of worker streams through gpgp_fit / gpgp_pred, overlapping on the
 * device. keep = 1 leaves the fitted model resident (its memory stays counted
 * against the budget) and returns its id for predict requests (model >= 0),
 * until gpgp_server_release. Outputs: mean / var (m doubles each, caller-owned
 * host memory that must stay valid until the request completes; var may be
 * NULL). A request's results do not depend on what else is in flight. */
typedef struct gpgp_server gpgp_server;
typedef struct gpgp_server_opts {
  int32_t device;
  int32_t workers;       /* worker streams for non-batched requests (default 4) */
  int64_t hbm_budget;    /* bytes for in-flight work and resident models (0: 80% of free) */
  int32_t precision;     /* GPGP_PREC_FP64 or GPGP_PREC_MIXED, for every request */
  int32_t batch_max_n;   /* largest n sent to the batch lane (default 1024, at most 4096) */
  int32_t batch_max;     /* most requests in one batch (default 4096) */
  double jitter;         /* added to K for every fit (default 1e-6 when <= 0) */
} gpgp_server_opts;
typedef struct gpgp_request {
  const gpgp_kernel *kernel;
  const gpgp_lik *lik;
  const gpgp_method *method;   /* NULL: method_full */
  const gpgp_approx *approx;   /* NULL: approx_laplace defaults */
  const double *x;             /* n-by-d column-major */
  int64_t n;
  int32_t d;
  const double *y, *trials, *offset; /* trials / offset may be NULL */
  const double *xt;            /* m-by-d column-major */
  int64_t m;
  int32_t keep;                /* keep the fitted model resident */
  int64_t model;               /* >= 0: predict with this resident model (fit fields unused) */
  double *mean, *var;          /* outputs, m doubles each (var may be NULL) */
} gpgp_request;
typedef struct gpgp_request_result {
  int32_t status;              /* gpgp_status of the request */
  int32_t lane;                /* 0 batch lane, 1 worker stream */
  double log_evidence;         /* fit requests */
  int32_t converged, iters;    /* of the Laplace / EP iteration (Gaussian: 1, 1) */
  int32_t precision_used;      /* as gpgp_fit_result.precision_used */
  int32_t reserved;
  int64_t model;               /* id of the resident model (keep = 1), else -1 */
  double queue_ms, run_ms, total_ms; /* admission wait, service, submit -> done */
} gpgp_request_result;
typedef struct gpgp_server_stats {
  int64_t submitted, completed, failed, pending, inflight;
  int64_t batches, batched_requests;
  int64_t bytes_inflight, bytes_resident, bytes_peak, budget;
  double p50_ms, p99_ms, max_ms; /* total latency of the completed requests */
} gpgp_server_stats;
gpgp_status gpgp_server_create(const gpgp_server_opts *opts, gpgp_server **out);
gpgp_status gpgp_server_submit(gpgp_server *s, const gpgp_request *req, int64_t *id);
/* GPGP_OK with *res filled once the request is done (the id is then retired),
 * GPGP_EBUSY while it is not after waiting up to wait_ms (< 0: until done). */
gpgp_status gpgp_server_poll(gpgp_server *s, int64_t id, int32_t wait_ms, gpgp_request_result *res);
gpgp_status gpgp_server_release(gpgp_server *s, int64_t model);
gpgp_status gpgp_server_stats_get(gpgp_server *s, gpgp_server_stats *out);
/* waits for every submitted request, then stops the lanes */
gpgp_status gpgp_server_destroy(gpgp_server *s);

/* ---- allocation-free Gaussian fit (no counterpart in the reference) ---
 * For callers that cannot allocate device memory while they need a fit: a
 * serving process whose own pool already owns all of HBM, a latency-critical
 * request path where an allocation stall or failure is not acceptable, or a
 * host framework that forbids allocation while it drives the GPU. Runs the
 * plain FP64 fit of gp_fit for lik_gaussian + method_full and writes alpha (n
 * doubles, device memory) and the log evidence (one double, host memory);
 * x (n-by-d column-major) and y are device memory owned by the caller.
 * All scratch lives in one fixed device array of the library (about 4.8 MB,
 * held by every GPU that loads the library until the process exits), so the
 * call never allocates. Limits: n <= 512 and at most 64 feature columns,
 * otherwise GPGP_EINVAL. The call makes the context's device current; its
 * first call for a device also looks up the array's device address, so make
 * that first call before any stream capture begins. Calls share the array:
 * calls whose GPU work overlaps race on it and must be serialised. Each call
 * waits for its own GPU work before it returns. Returns GPGP_ENAN (and a NaN
 * evidence) for NaN or Inf in x or y, GPGP_ENOT_PD (and -Inf) when the
 * factorisation fails. */
gpgp_status gpgp_fit_gaussian_noalloc(gpgp_ctx *ctx, const gpgp_kernel *k, double sigma,
                                      double jitter, const double *x, int64_t n, int32_t d,
                                      const double *y, double *alpha, double *log_evidence);

/* ---- self-test of the mixed-precision product: C = C - A B^T for random
 *      M x K and N x K operands with entries spread over 2^8 in magnitude,
 *      computed with the BF16-sliced tensor-core GEMM and with the FP64 GEMM;
 *      returns max |difference| / max |C|. slices is 4 (32-bit fixed point,
 *      the factorisation path) or 5 (40-bit, the batched path). ---- */
gpgp_status gpgp_mixed_selftest(gpgp_ctx *ctx, int64_t M, int64_t N, int64_t K, int32_t slices,
                                double *max_rel_err);

/* ---- self-test of the mixed-precision covariance: K(x, x) + jitter I and its
 *      derivative matrices for the energy gradient (lscale and magnitude slots),
 *      evaluated in double-float arithmetic (the mixed-precision fit's path for
 *      kernels of cf_const, cf_sexp, cf_matern32 and cf_matern52 terms) and with
 *      the FP64 kernels. x is n-by-d column-major (host). Returns in
 *      max_rel_err[0] the largest max |difference| / max |FP64 entry| over the
 *      lower triangles of K and of every derivative matrix, and in
 *      max_rel_err[1] the largest per-entry relative difference of K over its
 *      entries above 1e-20 of its maximum (smaller entries lose relative
 *      accuracy as the pair's low part leaves the FP32 normal range; their
 *      absolute error stays below 1e-35 of it). Derivative entries that vanish
 *      with the distance (lscale slots of nearly coincident points) carry the
 *      inputs' 48-bit representation error relative to that distance, so they
 *      are held in the max norm only. GPGP_EUNSUPPORTED for other kernels. No
 *      counterpart in the reference. ---- */
gpgp_status gpgp_cov_df_selftest(gpgp_ctx *ctx, const gpgp_kernel *k, const double *x, int64_t n, int32_t d,
                                 double jitter, double *max_rel_err);

/* ---- bounded-wait self-test: a kernel polls an mbarrier that nothing completes
 *      for `polls` iterations (the same loop as the tensor-core kernels' waits,
 *      whose bound is 2^24), records the timeout and returns; the call returns
 *      GPGP_ETIMEOUT and the context stays usable. ---- */
gpgp_status gpgp_wait_selftest(gpgp_ctx *ctx, int32_t polls);

#ifdef __cplusplus
}
#endif
#endif /* GPGP_H */
