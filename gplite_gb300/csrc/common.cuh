// Internal declarations shared by the libgpgp translation units.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <mutex>
#include <string>
#include <vector>

#include "gpgp.h"

namespace gpgp {

// ---------------------------------------------------------------------------
// error handling: every CUDA call is checked; failures turn into GPGP_ECUDA
// with the message kept on the context (never abort, never trap).
// ---------------------------------------------------------------------------
struct CudaError {
  cudaError_t err;
  const char *what;
  int line;
};

#define GPGP_CUDA(call)                                                   \
  do {                                                                    \
    cudaError_t e__ = (call);                                             \
    if (e__ != cudaSuccess) throw ::gpgp::CudaError{e__, #call, __LINE__}; \
  } while (0)

// Number of kernel launches issued through the library (all contexts and
// threads). Launches recorded into a graph under capture are not counted; a
// graph replay adds its kernel nodes.
extern std::atomic<int64_t> g_launches;
extern thread_local bool tl_capturing;
#define GPGP_LAUNCHED()                                                                 \
  do {                                                                                 \
    if (!::gpgp::tl_capturing) ::gpgp::g_launches.fetch_add(1, std::memory_order_relaxed); \
  } while (0)
// Per-kernel timers (gpgp_kernel_profile_read): the API entry points bind the
// context's timer to the calling thread while profiling is on; KTScope
// brackets one launch with events and adds its executed arithmetic.
struct KernelTimer {
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> ev;
  double ms[GPGP_NKPROF] = {0};
  double flops[GPGP_NKPROF] = {0};
  int64_t launches[GPGP_NKPROF] = {0};
  void collect();
  void reset();
};
extern thread_local KernelTimer *tl_kt;
struct KTScope {
  cudaStream_t s;
  int k;
  cudaEvent_t a = nullptr, b = nullptr;
  KTScope(int kernel, cudaStream_t st, double flops);
  ~KTScope();
};

#define GPGP_CHECK_LAUNCH()              \
  do {                                   \
    GPGP_LAUNCHED();                     \
    GPGP_CUDA(cudaPeekAtLastError());    \
  } while (0)

// A value computed once per device: function attributes (dynamic shared-memory
// limits) and device properties belong to the device that is current when
// they are set or read, so a process that drives several GPUs must set them
// on each. per_device(pd, fn) returns fn() for the current device, calling it
// at most once per device (devices >= 64 call it every time). Thread-safe.
struct PerDevice {
  std::mutex mu;
  uint64_t done = 0;
  int val[64] = {0};
};
template <class F>
int per_device(PerDevice &pd, F &&fn) {
  int dev = 0;
  GPGP_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return fn();
  std::lock_guard<std::mutex> g(pd.mu);
  if (!((pd.done >> dev) & 1ull)) {
    pd.val[dev] = fn();
    pd.done |= 1ull << dev;
  }
  return pd.val[dev];
}
// SMs of the current device (cached per device).
int device_sms();

// ---------------------------------------------------------------------------
// covariance program on the device
// ---------------------------------------------------------------------------
// Features: every term reads its own columns of a feature matrix F (rows =
// points, column-major with leading dimension ld). prep_features() writes
// them: the term's input columns (vars subset), normalised when asked; for a
// periodic term the columns are [sin(w x), cos(w x), x] with w = 2*pi/period.
struct DevTerm {
  int kind;      // gpgp_cf_kind of the (base) kernel
  int group;     // product group
  int periodic;  // 1: features are [sin, cos, raw]
  int off;       // first feature column of this term
  int nv;        // number of input columns used
  int dt;        // feature columns read by the kernel (nv, or 2*nv if periodic)
  double m2;     // magn^2
  double c1;     // sexp: 1/lscale^2; matern32/52: sqrt(3|5)/lscale; nn: sigma0^2*sigma^2
  double c2;     // nn: sigma^2; periodic: w = 2*pi/period
};

struct DevKernel {
  int nterms;
  int ngroups;
  int nfeat;     // total feature columns
  DevTerm t[GPGP_MAX_TERMS];
};

// Host-side description of where each term's inputs come from.
struct HostTermPrep {
  int nv;
  int vars[GPGP_MAX_VARS];
  int normalize;
  int periodic;
  double means[GPGP_MAX_VARS];
  double scales[GPGP_MAX_VARS];
  double w;
};

gpgp_status build_dev_kernel(const gpgp_kernel *k, int d, DevKernel *dk,
                             std::vector<HostTermPrep> *prep, std::string *err);

// Feature matrix F (n x nfeat, leading dimension ldf) from x (n x d, ldx).
void prep_features(cudaStream_t s, const DevKernel &dk, const std::vector<HostTermPrep> &prep,
                   const double *x, int64_t n, int64_t ldx, double *F, int64_t ldf);

// Output modes of the covariance tile generator.
enum CovMode {
  COV_FULL = 0,     // out = K(x1, x2) (+ jitter on the diagonal when sym)
  COV_B = 1,        // out = I + s_i s_j (K + jitter I)_ij  (lower triangle, sym only)
  COV_ROWSCALE = 2  // out_ij = s_i K(x1_i, x2_j) (cross, no jitter)
};

// out (n1 x n2, ldo). sym: x1 == x2 (only lower tiles evaluated; upper mirrored
// when mirror = 1). s: per-row scale (COV_B, COV_ROWSCALE) or null. err (device,
// optional): the feature tiles are staged by TMA bulk copies where they are
// aligned for it, and a bounded wait that runs out sets *err to 1; null: plain loads.
void cov_matrix(cudaStream_t s, const DevKernel &dk, uint32_t group_mask, const double *F1,
                int64_t ld1, int64_t n1, const double *F2, int64_t ld2, int64_t n2, double *out,
                int64_t ldo, int mode, int sym, int mirror, double jitter, const double *scale,
                int *err = nullptr);

// out[i] = K(x1_i, x2_i) for i < n (diagonal).
void cov_diag(cudaStream_t s, const DevKernel &dk, uint32_t group_mask, const double *F1,
              int64_t ld1, const double *F2, int64_t ld2, int64_t n, double *out);

// out[i] = sum_j K(x1_i, x2_j) v_j for i < n1 (fused, K never stored).
void cov_matvec(cudaStream_t s, const DevKernel &dk, uint32_t group_mask, const double *F1,
                int64_t ld1, int64_t n1, const double *F2, int64_t ld2, int64_t n2,
                const double *v, double *out);

// Gradient contraction: g[t*5 + p] = sum_{i,j} W_ij dK_ij / dlog(theta_{t,p}) over the
// symmetric W given by its lower triangle (ldw); partial sums per tile in part,
// reduced in a fixed order. Returns EUNSUPPORTED for parameters without a derivative.
gpgp_status cov_grad_contract(cudaStream_t s, const DevKernel &dk, const double *F, int64_t ldf,
                              int64_t n, const double *W, int64_t ldw, double *part, double *g);
int64_t cov_grad_partials(int64_t n);

// Derivative matrices of K written by the covariance pass when the energy
// gradient follows the fit (cov.cu). Matrix q is the value of product group
// a[q] (kind 0; every magnitude slot of the group is twice it) or the
// derivative of K with respect to slot b[q] of term a[q] (kind 1).
constexpr int GPGP_GRAD_MAXMAT = 8;
struct GradMats {
  int nmat;
  int kind[GPGP_GRAD_MAXMAT];
  int a[GPGP_GRAD_MAXMAT];
  int b[GPGP_GRAD_MAXMAT];
  int grp[GPGP_GRAD_MAXMAT];  // the product group of matrix q
};
// slot_mat[t*5 + p]: the slot's matrix (gradient = slot_scale x its sum), -1: a
// constant derivative (slot_scale x the sum of W), -2: not a parameter.
struct GradPlan {
  GradMats m;
  int slot_mat[GPGP_MAX_TERMS * GPGP_TERM_NPARAM];
  double slot_scale[GPGP_MAX_TERMS * GPGP_TERM_NPARAM];
};
// false: more than GPGP_GRAD_MAXMAT matrices would be needed.
bool plan_grad_store(const DevKernel &dk, GradPlan *pl);
// K (n x n, ldk, lower tiles mirrored, jitter on the diagonal) and the planned
// matrices D + q dstride (ldd; entries i >= j only), 64 x 64 tiles.
void cov_matrix_grad(cudaStream_t s, const DevKernel &dk, const GradPlan &pl, const double *F, int64_t ldf,
                     int64_t n, double *K, int64_t ldk, double jitter, double *D, int64_t ldd, int64_t dstride,
                     int *err = nullptr);
// g[q] = sum_ij W_ij D_q(i, j), g[nmat] = sum_ij W_ij, with W = alpha alpha^T -
// diag(s) Binv diag(s) formed on the fly from the lower triangle of Binv; df: in
// double-float arithmetic (mixed precision).
void grad_stored_contract(cudaStream_t s, const GradPlan &pl, int64_t n, const double *Bi, int64_t ldb,
                          const double *alpha, const double *sv, const double *D, int64_t ldd, int64_t dstride,
                          double *part, double *g, bool df = false);
int64_t grad_stored_partials(int64_t n);
// hg[t*5 + p] from the contraction's sums g (host).
void grad_stored_assemble(const GradPlan &pl, int nterms, const double *g, double *hg);
// Mixed precision: K (and with pl the planned derivative matrices) evaluated in
// double-float arithmetic on the FP32 pipe, for kernels of cf_const, cf_sexp,
// cf_matern32 and cf_matern52 terms without periodic inputs (cov_df_eligible).
bool cov_df_eligible(const DevKernel &dk);
// err (device) receives 1 when a bounded wait of the kernel's TMA staging ran out
// (null: plain loads). With B, the lower triangle of B = I + s2 K (ldb) as well.
void cov_matrix_df(cudaStream_t s, const DevKernel &dk, const GradPlan *pl, const double *F, int64_t ldf, int64_t n,
                   double *K, int64_t ldk, double jitter, double *D, int64_t ldd, int64_t dstride, int *err,
                   double *B = nullptr, int64_t ldb = 0, double s2 = 0.0);
// Mixed precision, the same kernels: out_ij = s_i K(x1_i, x2_j) (scale null: 1) and
// out_i = sum_j K(x1_i, x2_j) v_j over the groups of gmask, in double-float arithmetic.
void cov_cross_df(cudaStream_t s, const DevKernel &dk, uint32_t gmask, const double *F1, int64_t ld1, int64_t n1,
                  const double *F2, int64_t ld2, int64_t n2, double *out, int64_t ldo, const double *scale);
void cov_matvec_df(cudaStream_t s, const DevKernel &dk, uint32_t gmask, const double *F1, int64_t ld1, int64_t n1,
                   const double *F2, int64_t ld2, int64_t n2, const double *v, double *out);

// ---------------------------------------------------------------------------
// dense FP64 linear algebra (column-major)
// ---------------------------------------------------------------------------
constexpr int NB = 64;  // block size of the blocked factorisations
constexpr int DIAG_THREADS = 512;  // threads of the diagonal-block kernel (potrf_diag_kernel)

// C = alpha * op(A) op(B) + beta * C. lower_only: only tiles on/below the
// diagonal of C are computed (SYRK-style). tri_k: A and B are triangular so
// that terms with k < max(row, col) vanish (lauum of a lower factor).
void gemm64(cudaStream_t s, bool ta, bool tb, int64_t M, int64_t N, int64_t K, double alpha,
            const double *A, int64_t lda, const double *B, int64_t ldb, double beta, double *C,
            int64_t ldc, bool lower_only = false, int tri_mode = 0);

// Batched FP64 GEMM: problem z uses A + z sA, B + z sB, C + z sC.
void gemm64_batched(cudaStream_t s, bool ta, bool tb, int64_t M, int64_t N, int64_t K, double alpha,
                    const double *A, int64_t lda, int64_t sA, const double *B, int64_t ldb, int64_t sB,
                    double beta, double *C, int64_t ldc, int64_t sC, int64_t batch,
                    bool lower_only = false, int tri_mode = 0);
// Batched Cholesky of `batch` problems of equal size (see potrf).
void potrf_batched(cudaStream_t s, double *A, int64_t n, int64_t lda, int64_t sA, double *Winv,
                   int64_t sW, double *logdet_part, int64_t sL, int *status, int64_t batch);

// Blocked right-looking Cholesky of the lower triangle of A (n x n, lda), in
// place. Winv receives the inverses of the NB x NB diagonal factors
// (nblocks * NB * NB); logdet_part the per-block sums of log L_jj; status[0]
// the first failing pivot (1-based, 0 = OK). Later kernels of the same
// sequence see a non-zero status and return without work. panel_mode 0: the
// rows below each diagonal block by substitution (backward stable for an
// ill-conditioned block, e.g. FITC's K_z); 1: by the block's inverse, spread
// over many CTAs (for well-conditioned matrices such as B = I + S K S).
void potrf(cudaStream_t s, double *A, int64_t n, int64_t lda, double *Winv, double *logdet_part,
           int *status, int panel_mode = 0);

// Triangular solves with the blocked factor (lower L, diagonal inverses Winv).
// b is consumed as workspace; x receives the solution (x != b).
void trsv_lower(cudaStream_t s, const double *L, int64_t n, int64_t lda, const double *Winv,
                double *b, double *x, const int *status);    // x = L^-1 b
void trsv_lower_t(cudaStream_t s, const double *L, int64_t n, int64_t lda, const double *Winv,
                  double *b, double *x, const int *status);  // x = L^-T b
// Single-launch versions (blocks ordered by device flags, bounded waits): sync
// holds n / 64 + 2 unsigned words of device scratch; err is set when a wait runs
// out. b is not modified; x must not alias b.
void trsv_flow(cudaStream_t s, const double *L, int64_t n, int64_t lda, const double *Winv,
               const double *b, double *x, bool trans, const int *status, unsigned *sync, int *err);
// Substitution solves with a small lower factor L (M x M), as forwardsolve /
// backsolve: rows of the n x M matrix B (mode 0: X = B L^-T, mode 1: X = B L^-1),
// and vectors (x = L^-1 b, or L^-T b when trans).
void tri_rows(cudaStream_t s, const double *L, int64_t M, int64_t ldl, const double *B, int64_t ldb,
              double *X, int64_t ldx, int64_t n, int mode);
void tri_vec(cudaStream_t s, const double *L, int64_t M, int64_t ldl, const double *b, double *x,
             bool trans);
// B <- L^-1 B (n x m, ldb); tmp holds NB * m doubles.
void trsm_lower(cudaStream_t s, const double *L, int64_t n, int64_t lda, const double *Winv,
                double *B, int64_t m, int64_t ldb, double *tmp, const int *status);
// Wout = L^-1 (lower, strict upper = 0); tmp holds NB * n doubles.
void trtri_lower(cudaStream_t s, const double *L, int64_t n, int64_t lda, const double *Winv,
                 double *Wout, int64_t ldw, double *tmp, const int *status);
// out[j] = sum_i W_ij^2 (column norms of a lower-triangular W) = diag(W^T W).
void col_sumsq_lower(cudaStream_t s, const double *W, int64_t n, int64_t ldw, double *out);
// out[j] = sum_i B_ij^2 for an n x m dense B.
void col_sumsq(cudaStream_t s, const double *B, int64_t n, int64_t m, int64_t ldb, double *out);
// y = A x with symmetric A given by its full storage (n x n).
void gemv64(cudaStream_t s, bool trans, int64_t M, int64_t N, double alpha, const double *A,
            int64_t lda, const double *x, double beta, double *y);
// y = W x (trans false) or W^T x (trans true) for a lower-triangular W whose strict
// upper part is zero (n x n, ldw).
void trmv_lower(cudaStream_t s, bool trans, int64_t n, const double *W, int64_t ldw, const double *x, double *y);
// Sum of logdet partials (fixed order) -> out[0].
void sum_vec(cudaStream_t s, const double *v, int64_t n, double *out);
// LU with partial pivoting of a general n x n A (lda), in place; piv[k] is the row
// swapped with row k at step k; status[0] = k + 1 at an exactly zero pivot.
void getrf(cudaStream_t s, double *A, int64_t n, int64_t lda, int *piv, int *status);
// X <- A^-1 X (n x m, ldx) with the factors of getrf.
void getrs(cudaStream_t s, const double *LU, int64_t n, int64_t lda, const int *piv, double *X, int64_t m,
           int64_t ldx, const int *status);

// ---------------------------------------------------------------------------
// mixed precision (mixed.cu / mixed_la.cu): BF16-sliced operands for tcgen05
// ---------------------------------------------------------------------------
struct OzSplit {
  int *ex = nullptr;        // per-row power-of-two exponents (rows padded)
  uint16_t *sl = nullptr;   // BF16 slices, pre-tiled for UMMA
  int64_t rows = 0, K = 0, nrb = 0, nkb = 0;
  int64_t bstride_ex = 0, bstride_sl = 0;  // batched operands: per-problem strides
  int S = 4;  // slices (8S-bit fixed point); both operands of a product use the same S
};
int64_t oz_nrb(int64_t rows);
size_t oz_split_bytes(int64_t rows, int64_t K, int S = 4);
void oz_split_bind(void *mem, int64_t rows, int64_t K, OzSplit *out, int S = 4);
// rows x K operand: element (r, k) = P[r + k*ld] (trans 0) or P[k + r*ld] (trans 1)
void oz_split(cudaStream_t s, const double *P, int64_t ld, int trans, int64_t rows, int64_t K,
              OzSplit *out);
// C = alpha A B^T + beta C on K chunks [kc0, kc1) (64 wide); a_row0/b_row0 multiples of 64.
// kmode: 0 all chunks; 1 start at max(row, col); 2 start at col; 3 stop after row.
// status (optional): the launch is skipped for a problem whose word is nonzero; the
// word must not change while the launch runs (each role of a CTA reads it).
void oz_gemm(cudaStream_t s, const OzSplit &A, int64_t a_row0, const OzSplit &B, int64_t b_row0,
             int64_t M, int64_t N, int64_t kc0, int64_t kc1, int kmode, double alpha, double beta,
             double *C, int64_t ldc, bool lower_only, int *err, const int *status = nullptr);
// Grid cap of the sliced GEMM on this thread (0: one CTA per SM), for launches
// that share the GPU with work on another stream.
extern thread_local int tl_oz_grid_cap;
struct OzGridCap {
  int old;
  explicit OzGridCap(int cap) : old(tl_oz_grid_cap) { tl_oz_grid_cap = cap; }
  ~OzGridCap() { tl_oz_grid_cap = old; }
};
int oz_sms();  // SMs of the current device
// Two more streams with their events, owned by a context, for work that runs
// beside its main stream (the mixed Cholesky: s factors the diagonal chain of the
// next panel, s2 the panel's rows below it).
struct SideStream {
  cudaStream_t s = nullptr, s2 = nullptr;
  cudaEvent_t fork = nullptr, a = nullptr, l = nullptr, c = nullptr, b = nullptr;
};
// Batched versions: problem z uses P + z sP and the split's batch strides (set
// bstride_ex / bstride_sl before splitting); C + z sC; status + z status_bs.
void oz_split_batched(cudaStream_t s, const double *P, int64_t ld, int64_t sP, int trans, int64_t rows,
                      int64_t K, OzSplit *out, int64_t batch);
void oz_gemm_batched(cudaStream_t s, const OzSplit &A, int64_t a_row0, const OzSplit &B, int64_t b_row0,
                     int64_t M, int64_t N, int64_t kc0, int64_t kc1, int kmode, double alpha,
                     double beta, double *C, int64_t ldc, int64_t sC, bool lower_only, int *err,
                     const int *status, int64_t status_bs, int64_t batch);

// Mixed-precision factorisation and inverses (same outputs as the FP64 versions).
// With a side stream, panel p + 1 is factored on it while the main stream
// finishes the trailing update of panel p (identical results).
void potrf_mixed(cudaStream_t s, double *A, int64_t n, int64_t lda, double *Winv,
                 double *logdet_part, int *status, int *err, const SideStream *side = nullptr);
void trtri_mixed(cudaStream_t s, const double *L, int64_t n, int64_t lda, const double *Winv,
                 double *W, int64_t ldw, int *err);
// Binv (lower) = W^T W for lower-triangular W
void lauum_mixed(cudaStream_t s, const double *W, int64_t n, int64_t ldw, double *Binv,
                 int64_t ldb, int *err);
// T = W R (W lower n x n, R n x m), then out[j] = sum_i T_ij^2
void trmv_sumsq_mixed(cudaStream_t s, const double *W, int64_t n, int64_t ldw, const double *R,
                      int64_t m, int64_t ldr, double *out, int *err);

// ---------------------------------------------------------------------------
// likelihood kernels
// ---------------------------------------------------------------------------
struct LikDev {
  int kind, link;
  double sigma, phi;
};
// Laplace pseudo data (R/lik.R:188-201): z, V from f.
void lik_pseudodata_la(cudaStream_t s, const LikDev &lk, int64_t n, const double *f,
                       const double *y, const double *trials, const double *offset, double *z,
                       double *V);
// sum_i loglik(f_i) -> partial sums, reduced later
void lik_loglik(cudaStream_t s, const LikDev &lk, int64_t n, const double *f, const double *y,
                const double *trials, const double *offset, double *out_scalar, double *part);
// EP site update (R/lik.R:207-270) for all sites; writes z, V, logC, cavity
// moments; flags[0] |= 1 on NaN quadrature, flags[0] |= 2 on NaN sites.
void lik_ep_sites(cudaStream_t s, const LikDev &lk, int64_t n, int q, const double *ghx,
                  const double *ghw, const double *fmean, const double *fvar, const double *z_old,
                  const double *P_old, const double *y, const double *trials,
                  const double *offset, double damping, double *z, double *V, double *logC,
                  double *cav_mean, double *cav_var, int *flags);
// LOO log predictive densities by GH quadrature (R/gp_loo.R:90-96).
void lik_loo_gh(cudaStream_t s, const LikDev &lk, int64_t n, int q, const double *ghx,
                const double *ghw, const double *mean, const double *var, const double *y,
                const double *trials, const double *offset, double *loos);

// LOO densities by Monte Carlo with given standard normals z (n x draws,
// column-major) (R/gp_loo.R:97-103).
void lik_loo_mc(cudaStream_t s, const LikDev &lk, int64_t n, int64_t draws, const double *z, const double *mean,
                const double *var, const double *y, const double *trials, const double *offset, double *loos);

// Elementwise helpers.
void vec_axpby(cudaStream_t s, int64_t n, double a, const double *x, double b, double *y);
void vec_mul(cudaStream_t s, int64_t n, const double *a, const double *b, double *out);
void vec_rsqrt(cudaStream_t s, int64_t n, const double *v, double *out);  // 1/sqrt(v)
void dot_partial(cudaStream_t s, int64_t n, const double *a, const double *b, double *out);
void max_abs_diff(cudaStream_t s, int64_t n, const double *a, const double *b, double *out);

// GH nodes/weights of order q (R/quadrature.R:28-34), host computation.
void gauss_hermite(int q, std::vector<double> *x, std::vector<double> *w);

}  // namespace gpgp
