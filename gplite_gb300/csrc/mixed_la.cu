// Mixed-precision blocked algorithms built on the sliced tensor-core GEMM
// (mixed.cu): Cholesky, triangular inverse, B^-1 = L^-T L^-1 and the
// predictive-variance product. Outputs have the same meaning and layout as the
// FP64 routines of dense.cu; only the contractions change precision (products
// of 32-bit fixed-point row slices, accumulated exactly, summed in FP64).
//
// Cholesky is two-level right-looking: outer panels of NBO columns (384: faster
// at n = 16384 than 256 or 512), each factored with the 64-wide FP64 diagonal
// kernel of dense.cu, a sliced GEMM for the panel solve L21 = A21 W11^T and
// sliced GEMMs for the updates inside the panel; one sliced SYRK with K = NBO
// then updates the trailing matrix, so every trailing element is rewritten in
// FP64 once per outer panel.
#include <math.h>

#include <algorithm>
#include <vector>

#include "common.cuh"
#include "model.cuh"

namespace gpgp {

// potrf_diag_kernel and potrf_panel_inv_kernel live in dense.cu
__global__ void potrf_diag_kernel(double *__restrict__ A, int kb, int64_t lda,
                                  double *__restrict__ Winv, double *__restrict__ logdet_part,
                                  int *__restrict__ status, int64_t k0, int64_t sA, int64_t sW,
                                  int64_t sL);
__global__ void potrf_panel_inv_kernel(double *__restrict__ A21, int64_t m, int kb, int64_t lda,
                                       const double *__restrict__ W, const int *__restrict__ status);

namespace {

// Stream-ordered scratch for split operands (freed when the scope ends).
struct SplitBuf {
  void *p = nullptr;
  cudaStream_t s = nullptr;
  OzSplit sp;
  SplitBuf(cudaStream_t st, int64_t rows, int64_t K) : s(st) {
    const size_t b = oz_split_bytes(rows, K);
    if (cudaMallocAsync(&p, b, st) != cudaSuccess) {
      p = nullptr;
      (void)cudaGetLastError();
      throw std::bad_alloc();
    }
    oz_split_bind(p, rows, K, &sp);
  }
  ~SplitBuf() {
    if (p) cudaFreeAsync(p, s);
  }
};

#ifndef GPGP_NBO
#define GPGP_NBO 384
#endif
constexpr int64_t NBO = GPGP_NBO;  // outer panel width of the mixed Cholesky (a build-time tuning knob)
// Lookahead: a trailing update of at least LOOK_MIN_ROWS rows leaves LOOK_PANEL_SMS
// SMs to the next panel's factorisation, whose GEMMs are capped to them.
constexpr int64_t LOOK_MIN_ROWS = 6144;
constexpr int LOOK_PANEL_SMS = 32;

// The 64-wide blocks of the outer panel [k0, k0 + kbo). Only the panel's own rows
// lie on the chain from one diagonal block to the next, so they are kept apart:
//  - chain (stream x): the FP64 factor and inverse W of the diagonal block, the
//    block's rows inside the panel L_p = A_p W^T (FP64, by the inverse), and the
//    FP64 update of the rest of the panel's lower triangle by them;
//  - bulk (stream y, after the chain's block): the rows below the panel,
//    L_b = A_b W^T, and their update of the panel's remaining columns
//    A_b,rest -= L_b L_p^T, both sliced GEMMs.
// x and y may be the same stream (the single-stream schedule; same products in
// the same order, so the same factor). With two streams the bulk GEMMs take no
// status word: the chain's diagonal kernels may set it while they run.
void factor_panel(cudaStream_t x, cudaStream_t y, const SideStream *sd, double *A, int64_t n, int64_t lda,
                  double *Winv, double *logdet_part, int *status, int *err, int64_t k0, int64_t kbo, SplitBuf &a,
                  SplitBuf &w, SplitBuf &lp) {
  const bool two = x != y;
  const int64_t pend = k0 + kbo;  // first row / column after the panel
  const int64_t mb = n - pend;    // rows below the panel
  for (int64_t j0 = k0; j0 < pend; j0 += NB) {
    const int jb = (int)std::min<int64_t>(NB, pend - j0);
    const int64_t blk = j0 / NB;
    double *Wb = Winv + blk * NB * NB;
    {
      KTScope kts(GPGP_KPROF_POTRF_DIAG, x, 2.0 * jb * jb * jb / 3);
      potrf_diag_kernel<<<1, DIAG_THREADS, 0, x>>>(A + j0 + j0 * lda, jb, lda, Wb, logdet_part + blk, status, j0, 0,
                                                   0, 0);
    }
    GPGP_CHECK_LAUNCH();
    const int64_t mp = pend - (j0 + jb);  // panel rows below the block
    double *Ap = A + (j0 + jb) + j0 * lda;
    if (mp > 0) {
      potrf_panel_inv_kernel<<<(unsigned)((mp + 3) / 4), 256, 0, x>>>(Ap, mp, jb, lda, Wb, status);
      GPGP_CHECK_LAUNCH();
    }
    if (two) {
      GPGP_CUDA(cudaEventRecord(sd->c, x));
      GPGP_CUDA(cudaStreamWaitEvent(y, sd->c, 0));
    }
    if (mp > 0)
      gemm64(x, false, true, mp, mp, jb, -1.0, Ap, lda, Ap, lda, 1.0, A + (j0 + jb) + (j0 + jb) * lda, lda, true, 0);
    if (mb <= 0) continue;
    double *Ab = A + pend + j0 * lda;
    const int *sst = two ? nullptr : status;
    oz_split(y, Ab, lda, 0, mb, jb, &a.sp);
    oz_split(y, Wb, NB, 0, jb, jb, &w.sp);
    oz_gemm(y, a.sp, 0, w.sp, 0, mb, jb, 0, 1, 0, 1.0, 0.0, Ab, lda, false, err, sst);
    if (mp > 0) {
      oz_split(y, Ab, lda, 0, mb, jb, &a.sp);
      oz_split(y, Ap, lda, 0, mp, jb, &lp.sp);
      oz_gemm(y, a.sp, 0, lp.sp, 0, mb, mp, 0, 1, 0, -1.0, 1.0, A + pend + (j0 + jb) * lda, lda, false, err, sst);
    }
  }
  if (two) {  // the panel is complete on x once the bulk is
    GPGP_CUDA(cudaEventRecord(sd->b, y));
    GPGP_CUDA(cudaStreamWaitEvent(x, sd->b, 0));
  }
}

}  // namespace

void potrf_mixed(cudaStream_t s, double *A, int64_t n, int64_t lda, double *Winv,
                 double *logdet_part, int *status, int *err, const SideStream *side) {
  SplitBuf a(s, n, NBO);   // panel operand (rows below the current block)
  SplitBuf w(s, NB, NB);   // inverse of the diagonal block
  SplitBuf lp(s, NBO, NB);  // the block's rows inside the panel
  cudaStreamCaptureStatus cap_st = cudaStreamCaptureStatusNone;
  GPGP_CUDA(cudaStreamIsCapturing(s, &cap_st));
  // Per-kernel timers (tl_kt) time each launch alone, so a profiled call runs the
  // single-stream schedule.
  if (!side || !side->s || n <= 2 * NBO || cap_st != cudaStreamCaptureStatusNone || tl_kt) {
    for (int64_t k0 = 0; k0 < n; k0 += NBO) {
      const int64_t kbo = std::min<int64_t>(NBO, n - k0);
      factor_panel(s, s, nullptr, A, n, lda, Winv, logdet_part, status, err, k0, kbo, a, w, lp);
      const int64_t m2 = n - k0 - kbo;
      if (m2 > 0) {
        double *P = A + (k0 + kbo) + k0 * lda;
        oz_split(s, P, lda, 0, m2, kbo, &a.sp);
        oz_gemm(s, a.sp, 0, a.sp, 0, m2, m2, 0, (kbo + 63) / 64, 0, -1.0, 1.0,
                A + (k0 + kbo) + (k0 + kbo) * lda, lda, true, err, status);
      }
    }
    return;
  }
  // Lookahead. The side stream factors the panels; the main stream applies each
  // finished panel p to the next panel's columns first, releases the side stream
  // (event a), and then applies p to the rest of the trailing matrix while panel
  // p + 1 is factored beside it (the two touch disjoint columns). Every product
  // is the one the plain schedule computes, so the factor is the same.
  SplitBuf t(s, n, NBO);  // panel p as the trailing update's operand
  cudaStream_t x = side->s;
  GPGP_CUDA(cudaEventRecord(side->fork, s));
  GPGP_CUDA(cudaStreamWaitEvent(x, side->fork, 0));
  // The main stream waits for the side stream before the buffers above are freed,
  // also when an error leaves the loop early (destroyed before them).
  struct Join {
    const SideStream *sd;
    cudaStream_t main;
    ~Join() {
      if (sd->s2) {  // the bulk stream first (an error may leave the panel loop early)
        cudaEventRecord(sd->b, sd->s2);
        cudaStreamWaitEvent(sd->s, sd->b, 0);
      }
      cudaEventRecord(sd->l, sd->s);
      cudaStreamWaitEvent(main, sd->l, 0);
    }
  } join{side, s};
  const int sms = oz_sms();
  int panel_cap = 0;
  for (int64_t k0 = 0; k0 < n; k0 += NBO) {
    const int64_t kbo = std::min<int64_t>(NBO, n - k0);
    {
      OzGridCap cap(panel_cap);
      factor_panel(x, side->s2 ? side->s2 : x, side, A, n, lda, Winv, logdet_part, status, err, k0, kbo, a, w, lp);
    }
    GPGP_CUDA(cudaEventRecord(side->l, x));
    GPGP_CUDA(cudaStreamWaitEvent(s, side->l, 0));
    const int64_t m2 = n - k0 - kbo;
    if (m2 <= 0) break;
    double *P = A + (k0 + kbo) + k0 * lda;
    double *C = A + (k0 + kbo) + (k0 + kbo) * lda;
    oz_split(s, P, lda, 0, m2, kbo, &t.sp);
    const int64_t nb2 = std::min<int64_t>(NBO, m2);
    oz_gemm(s, t.sp, 0, t.sp, 0, m2, nb2, 0, (kbo + 63) / 64, 0, -1.0, 1.0, C, lda, true, err, status);
    GPGP_CUDA(cudaEventRecord(side->a, s));
    GPGP_CUDA(cudaStreamWaitEvent(x, side->a, 0));
    const int64_t m3 = m2 - nb2;
    panel_cap = 0;
    if (m3 > 0) {
      const bool share = m3 >= LOOK_MIN_ROWS && sms > 2 * LOOK_PANEL_SMS;
      if (share) panel_cap = LOOK_PANEL_SMS;
      OzGridCap cap(share ? sms - LOOK_PANEL_SMS : 0);
      // no status word: the side stream's diagonal kernels may set it while this
      // launch runs, and every role of a GEMM CTA must see the same value
      oz_gemm(s, t.sp, nb2, t.sp, nb2, m3, m3, 0, (kbo + 63) / 64, 0, -1.0, 1.0, C + nb2 + nb2 * lda, lda,
              true, err, nullptr);
    }
  }
}

// ---------------------------------------------------------------------------
// recursive triangular inverse: W = L^-1, W21 = -W22 (L21 W11)
// ---------------------------------------------------------------------------
// every 64 x 64 diagonal-block inverse into W's diagonal, one kernel
__global__ void put_diag_inverses_kernel(const double *__restrict__ Winv, int64_t n, double *__restrict__ W,
                                         int64_t ldw) {
  const int64_t blk = blockIdx.x, k0 = blk * NB;
  const int kb = (int)((n - k0) < NB ? (n - k0) : NB);
  const double *src = Winv + blk * NB * NB;
  for (int idx = threadIdx.x; idx < NB * NB; idx += blockDim.x) {
    const int r = idx % NB, c = idx / NB;
    if (r < kb && c < kb) W[(k0 + r) + (k0 + c) * ldw] = src[r + c * NB];
  }
}

constexpr int64_t TRTRI_BASE = 512;  // diagonal blocks inverted level by level, batched

// Batched scratch for a level: `count` split operands of rows x K each.
struct SplitBatch {
  void *p = nullptr;
  cudaStream_t s = nullptr;
  OzSplit sp;
  SplitBatch(cudaStream_t st, int64_t rows, int64_t K, int64_t count) : s(st) {
    const size_t per = (oz_split_bytes(rows, K) + 1023) / 1024 * 1024;
    if (cudaMallocAsync(&p, per * count, st) != cudaSuccess) {
      p = nullptr;
      (void)cudaGetLastError();
      throw std::bad_alloc();
    }
    oz_split_bind(p, rows, K, &sp);
    sp.bstride_ex = (int64_t)(per / sizeof(int));
    sp.bstride_sl = (int64_t)(per / sizeof(uint16_t));
  }
  ~SplitBatch() {
    if (p) cudaFreeAsync(p, s);
  }
};

// One level of the blocked inverse for every full b x b diagonal block at
// offsets k b (k < count), whose two halves are already inverted:
// W21 = -W22 (L21 W11), all blocks of the level in two batched GEMMs.
static void trtri_level(cudaStream_t s, const double *L, int64_t lda, double *W, int64_t ldw, int64_t b,
                        int64_t count, double *T, int *err) {
  const int64_t h = b / 2;
  {
    SplitBatch a(s, h, h, count), bb(s, h, h, count);
    oz_split_batched(s, L + h, lda, b * (lda + 1), 0, h, h, &a.sp, count);
    oz_split_batched(s, W, ldw, b * (ldw + 1), 1, h, h, &bb.sp, count);
    oz_gemm_batched(s, a.sp, 0, bb.sp, 0, h, h, 0, bb.sp.nkb, 2, 1.0, 0.0, T, h, h * h, false, err, nullptr, 0,
                    count);
  }
  {
    SplitBatch a(s, h, h, count), bb(s, h, h, count);
    oz_split_batched(s, W + h + h * ldw, ldw, b * (ldw + 1), 0, h, h, &a.sp, count);
    oz_split_batched(s, T, h, h * h, 1, h, h, &bb.sp, count);
    oz_gemm_batched(s, a.sp, 0, bb.sp, 0, h, h, 0, a.sp.nkb, 3, -1.0, 0.0, W + h, ldw, b * (ldw + 1), false, err,
                    nullptr, 0, count);
  }
}

// recursive triangular inverse: W = L^-1, W21 = -W22 (L21 W11). Nodes already
// inverted (64-blocks from the factorisation, and full aligned 128 / 256 / 512
// blocks from the batched levels) are skipped; above the base the split points
// are multiples of the base so that its blocks line up.
static void trtri_rec(cudaStream_t s, const double *L, int64_t n, int64_t lda, int64_t off, int64_t ntot,
                      double *W, int64_t ldw, double *T, int *err) {
  if (n <= NB) return;
  if ((n == 128 || n == 256 || n == TRTRI_BASE) && off % n == 0 && off + n <= ntot) return;
  const int64_t g = n > TRTRI_BASE ? TRTRI_BASE : NB;
  const int64_t n1 = ((n / 2) + g - 1) / g * g;
  const int64_t n2 = n - n1;
  trtri_rec(s, L, n1, lda, off, ntot, W, ldw, T, err);
  trtri_rec(s, L + n1 + n1 * lda, n2, lda, off + n1, ntot, W + n1 + n1 * ldw, ldw, T, err);
  // T = L21 W11  (n2 x n1): A = L21 (rows n2, K n1), B rows j = columns of W11 (W11[k, j], k >= j)
  {
    SplitBuf a(s, n2, n1), b(s, n1, n1);
    oz_split(s, L + n1, lda, 0, n2, n1, &a.sp);
    oz_split(s, W, ldw, 1, n1, n1, &b.sp);
    oz_gemm(s, a.sp, 0, b.sp, 0, n2, n1, 0, b.sp.nkb, 2, 1.0, 0.0, T, n2, false, err);
  }
  // W21 = -W22 T  (n2 x n1): A = W22 (rows n2, K n2, lower: k <= i), B rows j = columns of T
  {
    SplitBuf a(s, n2, n2), b(s, n1, n2);
    oz_split(s, W + n1 + n1 * ldw, ldw, 0, n2, n2, &a.sp);
    oz_split(s, T, n2, 1, n1, n2, &b.sp);
    oz_gemm(s, a.sp, 0, b.sp, 0, n2, n1, 0, a.sp.nkb, 3, -1.0, 0.0, W + n1, ldw, false, err);
  }
}

__global__ void zero_upper_kernel(double *W, int64_t n, int64_t ldw) {
  for (int64_t j = blockIdx.y; j < n; j += gridDim.y)
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < j;
         i += (int64_t)gridDim.x * blockDim.x)
      W[i + j * ldw] = 0.0;
}

void trtri_mixed(cudaStream_t s, const double *L, int64_t n, int64_t lda, const double *Winv,
                 double *W, int64_t ldw, int *err) {
  if (n <= 0) return;
  dim3 g((unsigned)std::min<int64_t>((n + 255) / 256, 64), (unsigned)std::min<int64_t>(n, 65535));
  zero_upper_kernel<<<g, 256, 0, s>>>(W, n, ldw);
  GPGP_CHECK_LAUNCH();
  put_diag_inverses_kernel<<<(unsigned)((n + NB - 1) / NB), 256, 0, s>>>(Winv, n, W, ldw);
  GPGP_CHECK_LAUNCH();
  double *T = nullptr;
  const int64_t h = (n / 2 + TRTRI_BASE) * (n / 2 + TRTRI_BASE);
  if (cudaMallocAsync((void **)&T, (size_t)h * sizeof(double), s) != cudaSuccess) {
    (void)cudaGetLastError();
    throw std::bad_alloc();
  }
  try {
    // the full aligned diagonal blocks of 128, 256 and 512, all blocks of a size at once
    for (int64_t b = 2 * NB; b <= TRTRI_BASE; b *= 2)
      if (n / b > 0) trtri_level(s, L, lda, W, ldw, b, n / b, T, err);
    trtri_rec(s, L, n, lda, 0, n, W, ldw, T, err);
  } catch (...) {
    cudaFreeAsync(T, s);
    throw;
  }
  GPGP_CUDA(cudaFreeAsync(T, s));
}

void lauum_mixed(cudaStream_t s, const double *W, int64_t n, int64_t ldw, double *Binv,
                 int64_t ldb, int *err) {
  // Binv_ij = sum_k W_ki W_kj (k >= max(i, j)); operand rows = columns of W
  SplitBuf a(s, n, n);
  oz_split(s, W, ldw, 1, n, n, &a.sp);
  oz_gemm(s, a.sp, 0, a.sp, 0, n, n, 0, a.sp.nkb, 1, 1.0, 0.0, Binv, ldb, true, err);
}

void trmv_sumsq_mixed(cudaStream_t s, const double *W, int64_t n, int64_t ldw, const double *R,
                      int64_t m, int64_t ldr, double *out, int *err) {
  // T = W R (n x m): A = W (rows n, K n, k <= i), B rows j = columns of R
  double *T = nullptr;
  if (cudaMallocAsync((void **)&T, (size_t)n * m * sizeof(double), s) != cudaSuccess) {
    (void)cudaGetLastError();
    throw std::bad_alloc();
  }
  {
    SplitBuf a(s, n, n), b(s, m, n);
    oz_split(s, W, ldw, 0, n, n, &a.sp);
    oz_split(s, R, ldr, 1, m, n, &b.sp);
    oz_gemm(s, a.sp, 0, b.sp, 0, n, m, 0, a.sp.nkb, 3, 1.0, 0.0, T, n, false, err);
  }
  col_sumsq(s, T, n, m, n, out);
  GPGP_CUDA(cudaFreeAsync(T, s));
}

}  // namespace gpgp

// ---------------------------------------------------------------------------
// self-test entry point: sliced GEMM against the FP64 GEMM on random data
// ---------------------------------------------------------------------------
namespace {
__global__ void fill_random_kernel(double *a, int64_t n, uint64_t seed, double scale_spread) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    uint64_t z = seed + 0x9E3779B97F4A7C15ull * (uint64_t)(i + 1);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    const double u = (double)(z >> 11) * (1.0 / 9007199254740992.0) - 0.5;
    // entries of varying magnitude exercise the per-row scaling
    const double mag = exp2(scale_spread * (double)((z >> 3) & 7) / 7.0 - scale_spread / 2);
    a[i] = u * mag;
  }
}

__global__ void max_abs_kernel(const double *a, const double *b, int64_t n, double *out) {
  __shared__ double sd[256], sm[256];
  double d = 0.0, m = 0.0;
  for (int64_t i = threadIdx.x; i < n; i += 256) {
    d = fmax(d, fabs(a[i] - b[i]));
    m = fmax(m, fabs(b[i]));
  }
  sd[threadIdx.x] = d;
  sm[threadIdx.x] = m;
  __syncthreads();
  for (int st = 128; st > 0; st >>= 1) {
    if (threadIdx.x < st) {
      sd[threadIdx.x] = fmax(sd[threadIdx.x], sd[threadIdx.x + st]);
      sm[threadIdx.x] = fmax(sm[threadIdx.x], sm[threadIdx.x + st]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[0] = sd[0];
    out[1] = sm[0];
  }
}
}  // namespace

extern "C" gpgp_status gpgp_mixed_selftest(gpgp_ctx *ctx, int64_t M, int64_t N, int64_t K,
                                           int32_t slices, double *max_rel_err) {
  using namespace gpgp;
  if (!ctx || M < 1 || N < 1 || K < 1 || !max_rel_err || (slices != 4 && slices != 5))
    return GPGP_EINVAL;
  cudaStream_t s = (cudaStream_t)gpgp_stream(ctx);
  KTBind bind(ctx);
  try {
    double *A = nullptr, *B = nullptr, *C1 = nullptr, *C2 = nullptr, *red = nullptr;
    int *err = nullptr;
    GPGP_CUDA(cudaMallocAsync((void **)&A, M * K * sizeof(double), s));
    GPGP_CUDA(cudaMallocAsync((void **)&B, N * K * sizeof(double), s));
    GPGP_CUDA(cudaMallocAsync((void **)&C1, M * N * sizeof(double), s));
    GPGP_CUDA(cudaMallocAsync((void **)&C2, M * N * sizeof(double), s));
    GPGP_CUDA(cudaMallocAsync((void **)&red, 4 * sizeof(double), s));
    GPGP_CUDA(cudaMallocAsync((void **)&err, sizeof(int), s));
    GPGP_CUDA(cudaMemsetAsync(err, 0, sizeof(int), s));
    fill_random_kernel<<<256, 256, 0, s>>>(A, M * K, 12345, 8.0);
    fill_random_kernel<<<256, 256, 0, s>>>(B, N * K, 777, 8.0);
    fill_random_kernel<<<256, 256, 0, s>>>(C1, M * N, 99, 0.0);
    GPGP_CUDA(cudaMemcpyAsync(C2, C1, M * N * sizeof(double), cudaMemcpyDeviceToDevice, s));
    {
      void *pa = nullptr, *pb = nullptr;
      GPGP_CUDA(cudaMallocAsync(&pa, oz_split_bytes(M, K, slices), s));
      GPGP_CUDA(cudaMallocAsync(&pb, oz_split_bytes(N, K, slices), s));
      OzSplit sa, sb;
      oz_split_bind(pa, M, K, &sa, slices);
      oz_split_bind(pb, N, K, &sb, slices);
      oz_split(s, A, M, 0, M, K, &sa);
      oz_split(s, B, N, 0, N, K, &sb);
      // C1 = -A B^T + C1 (sliced) ; C2 = -A B^T + C2 (FP64)
      oz_gemm(s, sa, 0, sb, 0, M, N, 0, sa.nkb, 0, -1.0, 1.0, C1, M, false, err);
      gemm64(s, false, true, M, N, K, -1.0, A, M, B, N, 1.0, C2, M);
      max_abs_kernel<<<1, 256, 0, s>>>(C1, C2, M * N, red);
      cudaFreeAsync(pa, s);
      cudaFreeAsync(pb, s);
    }
    double h[2];
    int herr = 0;
    GPGP_CUDA(cudaMemcpyAsync(h, red, 2 * sizeof(double), cudaMemcpyDeviceToHost, s));
    GPGP_CUDA(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, s));
    GPGP_CUDA(cudaStreamSynchronize(s));
    cudaFreeAsync(A, s);
    cudaFreeAsync(B, s);
    cudaFreeAsync(C1, s);
    cudaFreeAsync(C2, s);
    cudaFreeAsync(red, s);
    cudaFreeAsync(err, s);
    GPGP_CUDA(cudaStreamSynchronize(s));
    *max_rel_err = h[0] / (h[1] > 0 ? h[1] : 1.0);
    if (herr) return GPGP_ETIMEOUT;
    return GPGP_OK;
  } catch (const CudaError &e) {
    (void)cudaGetLastError();
    return fail(ctx, GPGP_ECUDA, std::string("CUDA error ") + cudaGetErrorString(e.err) + " in " + e.what);
  } catch (const std::bad_alloc &) {
    return GPGP_EOOM;
  }
}
