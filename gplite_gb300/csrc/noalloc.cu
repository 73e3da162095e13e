// Allocation-free Gaussian fit.
//
// Some callers cannot allocate device memory when they need a fit: a serving
// process that has already handed all of HBM to its own memory pool, a
// latency-critical request path where a cudaMalloc stall or failure is not
// acceptable, or a host framework that forbids allocation while it drives the
// GPU. gpgp_fit_gaussian_noalloc serves them: it runs the FP64 plain fit of
// gp_fit for lik_gaussian + method_full (covariance, blocked Cholesky of
// B = I + K / sigma^2, solves, log evidence) with every intermediate in one
// file-scope device array of fixed size, and calls no allocating routine.
//
// Limits and rules:
//  - n <= 512 and at most 64 feature columns; larger
//    requests are rejected with GPGP_EINVAL.
//  - The array is a host-side stand-in in host code; its device address is
//    looked up once per device with cudaGetSymbolAddress, on the first call
//    made for that device (the call makes the context's device current
//    first). Make that first call before any stream capture begins.
//  - Every call on a device shares the one array and leaves its contents
//    behind. Calls whose GPU work overlaps (two streams, two host threads)
//    race on it; serialise them. Each call waits for its own GPU work before
//    it returns.
//  - Every GPU that loads the library holds the array (about 4.8 MB) until the
//    process exits.
#include <math.h>

#include <mutex>

#include "common.cuh"
#include "model.cuh"

namespace gpgp {
namespace {

constexpr int64_t NA_MAX_N = 512;
constexpr int64_t NA_MAX_FEAT = 64;
constexpr int64_t NA_NBLK = NA_MAX_N / NB;
// layout of the scratch array (doubles)
constexpr int64_t NA_K = 0;                                   // covariance, n x n
constexpr int64_t NA_L = NA_K + NA_MAX_N * NA_MAX_N;          // factor of B, n x n
constexpr int64_t NA_WINV = NA_L + NA_MAX_N * NA_MAX_N;       // inverses of the diagonal blocks
constexpr int64_t NA_F = NA_WINV + NA_NBLK * NB * NB;         // features, n x nfeat
constexpr int64_t NA_VEC = NA_F + NA_MAX_N * NA_MAX_FEAT;     // 6 vectors of n
constexpr int64_t NA_RED = NA_VEC + 6 * NA_MAX_N;             // reductions
constexpr int64_t NA_TOTAL = NA_RED + 512;
constexpr int64_t NA_INTS = 8;  // status words: [0] factorisation, [1] non-finite input

static __device__ __align__(256) double g_noalloc_scratch[NA_TOTAL];
static __device__ __align__(256) int g_noalloc_status[NA_INTS];

struct NoallocPtrs {
  double *scratch = nullptr;
  int *status = nullptr;
};

std::mutex g_na_mu;
NoallocPtrs g_na_ptrs[64];

// Device addresses of the arrays on `device`, which must be current (looked up
// once per device).
gpgp_status noalloc_setup(int device, NoallocPtrs *out, std::string *err) {
  if (device < 0 || device >= 64) {
    *err = "device index out of range";
    return GPGP_EINVAL;
  }
  std::lock_guard<std::mutex> g(g_na_mu);
  NoallocPtrs &p = g_na_ptrs[device];
  if (!p.scratch) {
    cudaError_t e1 = cudaGetSymbolAddress((void **)&p.scratch, g_noalloc_scratch);
    cudaError_t e2 = cudaGetSymbolAddress((void **)&p.status, g_noalloc_status);
    if (e1 != cudaSuccess || e2 != cudaSuccess) {
      p.scratch = nullptr;
      p.status = nullptr;
      *err = std::string("cudaGetSymbolAddress failed: ") +
             cudaGetErrorString(e1 != cudaSuccess ? e1 : e2);
      return GPGP_ECUDA;
    }
  }
  *out = p;
  return GPGP_OK;
}

// B = I + K / sigma^2 on the lower triangle (R/laplace.R:27 with V = sigma^2):
// the same expression as the general path, s_i (K_ij s_j) + delta_ij, s = 1/sigma
__global__ void na_make_B(const double *__restrict__ K, int64_t n, double s,
                          double *__restrict__ B) {
  const int64_t j = blockIdx.y;
  for (int64_t i = j + threadIdx.x; i < n; i += blockDim.x) {
    const double v = s * (K[i + j * n] * s);
    B[i + j * n] = (i == j) ? 1.0 + v : v;
  }
}

__global__ void na_scale(int64_t n, double a, const double *__restrict__ x, double *__restrict__ y) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = a * x[i];
}

// fhat = K alpha = y - sigma^2 alpha for the Gaussian likelihood (C alpha = y)
__global__ void na_fhat(int64_t n, double s2, const double *__restrict__ y,
                        const double *__restrict__ alpha, double *__restrict__ f) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) f[i] = y[i] - s2 * alpha[i];
}

// flag |= 1 when any of v[0..n) is NaN or +-Inf
__global__ void na_nonfinite(int64_t n, const double *__restrict__ v, int *__restrict__ flag) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    if (!isfinite(v[i])) atomicOr(flag, 1);
}

// LML = loglik - 0.5 f^T alpha - 0.5 (2 sum log L_ii)  (R/laplace.R:33-38)
__global__ void na_lml(const double *__restrict__ ll, const double *__restrict__ fa,
                       const double *__restrict__ ld, double *__restrict__ out) {
  if (threadIdx.x == 0) out[0] = ll[0] - 0.5 * fa[0] - 0.5 * (2.0 * ld[0]);
}

}  // namespace
}  // namespace gpgp

using namespace gpgp;

extern "C" gpgp_status gpgp_fit_gaussian_noalloc(gpgp_ctx *ctx, const gpgp_kernel *k, double sigma,
                                                 double jitter, const double *x, int64_t n,
                                                 int32_t d, const double *y, double *alpha,
                                                 double *log_evidence) {
  if (!ctx) return GPGP_EINVAL;
  return guarded(ctx, [&]() -> gpgp_status {
    if (!k || !x || !y || !alpha || !log_evidence || n < 1 || d < 1 || !(sigma > 0))
      return fail(ctx, GPGP_EINVAL, "invalid argument");
    if (n > NA_MAX_N)
      return fail(ctx, GPGP_EINVAL, "n exceeds the fixed scratch of the allocation-free fit (n <= 512)");
    GPGP_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    NoallocPtrs P;
    std::string err;
    gpgp_status st = noalloc_setup(ctx->device, &P, &err);
    if (st != GPGP_OK) return fail(ctx, st, err);
    DevKernel dk;
    std::vector<HostTermPrep> prep;
    st = build_dev_kernel(k, d, &dk, &prep, &err);
    if (st != GPGP_OK) return fail(ctx, st, err);
    if (dk.nfeat > NA_MAX_FEAT)
      return fail(ctx, GPGP_EINVAL, "more than 64 feature columns for the allocation-free fit");
    double *K = P.scratch + NA_K, *Lf = P.scratch + NA_L, *Winv = P.scratch + NA_WINV;
    double *F = P.scratch + NA_F, *vec = P.scratch + NA_VEC, *red = P.scratch + NA_RED;
    double *t1 = vec, *t2 = vec + NA_MAX_N, *fh = vec + 2 * NA_MAX_N;
    int *status = P.status;
    // the factorisation reads status[0] and the input check ORs into status[1]:
    // both must start at zero (the array keeps the previous call's words)
    GPGP_CUDA(cudaMemsetAsync(status, 0, NA_INTS * sizeof(int), s));
    na_nonfinite<<<(unsigned)(((int64_t)n * d + 255) / 256), 256, 0, s>>>((int64_t)n * d, x, status + 1);
    GPGP_CHECK_LAUNCH();
    na_nonfinite<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, y, status + 1);
    GPGP_CHECK_LAUNCH();
    prep_features(s, dk, prep, x, n, n, F, n);
    cov_matrix(s, dk, 0xffffffffu, F, n, n, F, n, n, K, n, COV_FULL, 1, 1, jitter, nullptr);
    const double sinv = sqrt(1.0 / (sigma * sigma));
    na_make_B<<<dim3(1, (unsigned)n), 256, 0, s>>>(K, n, sinv, Lf);
    GPGP_CHECK_LAUNCH();
    double *logdet_part = red + 300;  // NA_NBLK + 1 slots
    potrf(s, Lf, n, n, Winv, logdet_part, status);
    // alpha = s L^-T L^-1 (s y)
    na_scale<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, sinv, y, t1);
    GPGP_CHECK_LAUNCH();
    trsv_lower(s, Lf, n, n, Winv, t1, t2, status);
    trsv_lower_t(s, Lf, n, n, Winv, t2, t1, status);
    na_scale<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, sinv, t1, alpha);
    GPGP_CHECK_LAUNCH();
    na_fhat<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, sigma * sigma, y, alpha, fh);
    GPGP_CHECK_LAUNCH();
    LikDev lk;
    lk.kind = GPGP_LIK_GAUSSIAN;
    lk.link = GPGP_LINK_IDENTITY;
    lk.sigma = sigma;
    lk.phi = 0.0;
    lik_loglik(s, lk, n, fh, y, nullptr, nullptr, red + 200, red);  // partials red[0..63]
    dot_partial(s, n, fh, alpha, red + 100);                        // result at red[164]
    sum_vec(s, logdet_part, (n + NB - 1) / NB, red + 250);
    na_lml<<<1, 32, 0, s>>>(red + 200, red + 164, red + 250, red + 260);
    GPGP_CHECK_LAUNCH();
    int hstatus[2] = {0, 0};
    GPGP_CUDA(cudaMemcpyAsync(hstatus, status, 2 * sizeof(int), cudaMemcpyDeviceToHost, s));
    GPGP_CUDA(cudaMemcpyAsync(log_evidence, red + 260, sizeof(double), cudaMemcpyDeviceToHost, s));
    GPGP_CUDA(cudaStreamSynchronize(s));
    if (hstatus[1] != 0) {
      *log_evidence = NAN;
      return fail(ctx, GPGP_ENAN, "x or y holds NaN or Inf");
    }
    if (hstatus[0] != 0) {
      *log_evidence = -INFINITY;
      return fail(ctx, GPGP_ENOT_PD, "Cholesky factorisation: matrix is not positive definite");
    }
    return GPGP_OK;
  });
}
