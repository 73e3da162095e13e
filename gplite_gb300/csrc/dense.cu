// Dense FP64 linear algebra for the GP hot path (column-major, lower factors).
//
// Replaces the LAPACK/BLAS calls the reference makes from R: chol (dpotrf,
// R/laplace.R:28, R/ep.R:38, R/linear_algebra.R:28), forwardsolve/backsolve
// (dtrsv/dtrsm, R/laplace.R:29, R/gp_pred.R:218) and %*% (dgemm/dgemv,
// R/laplace.R:30, R/gp_pred.R:209).
//
// The factorisation is blocked right-looking with NB = 64: the diagonal block
// is factored by one CTA in shared memory, which also inverts it (the inverses
// serve the solves); the panel below is solved by row-parallel substitution,
// which stays backward stable when a diagonal block is ill-conditioned (FITC's
// K_z); the trailing update is a lower-only GEMM on the FP64 pipe. The
// triangular solves are single launches ordered by per-block flags.
#include <math.h>

#include <algorithm>

#include "common.cuh"
#include "fp64math.cuh"

namespace gpgp {

// ---------------------------------------------------------------------------
// FP64 GEMM: C = alpha op(A) op(B) + beta C, 64x64 tiles, 4x4 per thread
// ---------------------------------------------------------------------------
constexpr int GBM = 64, GBN = 64, GBK = 16;

template <bool TA, bool TB>
__global__ void __launch_bounds__(256) gemm64_kernel(int64_t M, int64_t N, int64_t K, double alpha,
                                                     const double *__restrict__ A, int64_t lda,
                                                     const double *__restrict__ B, int64_t ldb,
                                                     double beta, double *__restrict__ C,
                                                     int64_t ldc, int lower_only, int tri_mode,
                                                     int64_t sA, int64_t sB, int64_t sC, int64_t kchunk) {
  const int64_t bm = blockIdx.x, bn = blockIdx.y;
  // blockIdx.z: the problem of a batch (strides sA, sB, sC), or with kchunk > 0 the
  // K range [z kchunk, (z + 1) kchunk) of one product whose partial goes to C + z sC
  A += blockIdx.z * sA;
  B += blockIdx.z * sB;
  C += blockIdx.z * sC;
  int64_t kend = K;
  const int64_t row0 = bm * GBM, col0 = bn * GBN;
  if (lower_only && col0 > row0 + GBM - 1) return;
  __shared__ double As[GBK][GBM + 1];
  __shared__ double Bs[GBK][GBN + 1];
  const int tid = threadIdx.x;
  const int tx = tid % 16, ty = tid / 16;
  double acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) acc[a][b] = 0.0;
  int64_t kstart = 0;
  if (tri_mode == 1) kstart = (row0 / GBK) * GBK;  // W^T W with W lower: k >= row
  if (kchunk > 0) {
    const int64_t kb = (int64_t)blockIdx.z * kchunk;
    kstart = kstart > kb ? kstart : kb;
    kend = kb + kchunk < K ? kb + kchunk : K;
  }
  for (int64_t k0 = kstart; k0 < kend; k0 += GBK) {
    // load A tile: op(A) is M x K
#pragma unroll
    for (int e = 0; e < (GBM * GBK) / 256; ++e) {
      int idx = tid + e * 256;
      int r, kk;
      if (!TA) {
        r = idx % GBM;
        kk = idx / GBM;
      } else {
        kk = idx % GBK;
        r = idx / GBK;
      }
      int64_t gr = row0 + r, gk = k0 + kk;
      double v = 0.0;
      if (gr < M && gk < kend) v = TA ? A[gk + gr * lda] : A[gr + gk * lda];
      As[kk][r] = v;
    }
    // load B tile: op(B) is K x N
#pragma unroll
    for (int e = 0; e < (GBN * GBK) / 256; ++e) {
      int idx = tid + e * 256;
      int c, kk;
      if (!TB) {
        kk = idx % GBK;
        c = idx / GBK;
      } else {
        c = idx % GBN;
        kk = idx / GBN;
      }
      int64_t gc = col0 + c, gk = k0 + kk;
      double v = 0.0;
      if (gc < N && gk < kend) v = TB ? B[gc + gk * ldb] : B[gk + gc * ldb];
      Bs[kk][c] = v;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < GBK; ++kk) {
      double a[4], b[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        a[q] = As[kk][tx + 16 * q];
        b[q] = Bs[kk][ty + 16 * q];
      }
#pragma unroll
      for (int p = 0; p < 4; ++p)
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[p][q] = fma(a[p], b[q], acc[p][q]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int p = 0; p < 4; ++p) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      int64_t r = row0 + tx + 16 * p, c = col0 + ty + 16 * q;
      if (r < M && c < N && (!lower_only || r >= c)) {
        double *dst = C + r + c * ldc;
        *dst = (beta == 0.0) ? alpha * acc[p][q] : alpha * acc[p][q] + beta * *dst;
      }
    }
  }
}

// C = alpha sum_z P_z + beta C over the split-K partials (fixed order)
__global__ void splitk_reduce_kernel(int64_t M, int64_t N, int nz, const double *__restrict__ P,
                                     double alpha, double beta, double *__restrict__ C, int64_t ldc,
                                     int lower_only) {
  const int64_t MN = M * N;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < MN;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = idx % M, c = idx / M;
    if (lower_only && r < c) continue;
    double s = 0.0;
    for (int z = 0; z < nz; ++z) s += P[idx + z * MN];
    double *dst = C + r + c * ldc;
    *dst = (beta == 0.0) ? alpha * s : alpha * s + beta * *dst;
  }
}

template <bool TA, bool TB>
static void launch_gemm64(cudaStream_t s, dim3 grid, int64_t M, int64_t N, int64_t K, double alpha,
                          const double *A, int64_t lda, const double *B, int64_t ldb, double beta, double *C,
                          int64_t ldc, int lo, int tri_mode, int64_t sA, int64_t sB, int64_t sC, int64_t kchunk) {
  double fl = 0.0;
  if (tl_kt) {  // executed FP64 arithmetic of the tiles this launch runs
    for (int64_t bm = 0; bm < (int64_t)grid.x; ++bm)
      for (int64_t bn = 0; bn < (int64_t)grid.y; ++bn) {
        const int64_t row0 = bm * GBM, col0 = bn * GBN;
        if (lo && col0 > row0 + GBM - 1) continue;
        const int64_t ks = tri_mode == 1 ? (row0 / GBK) * GBK : 0;
        fl += 2.0 * GBM * GBN * (double)std::max<int64_t>(0, K - ks);
      }
    if (kchunk == 0) fl *= (double)grid.z;
  }
  KTScope kts(GPGP_KPROF_GEMM64, s, fl);
  gemm64_kernel<TA, TB><<<grid, 256, 0, s>>>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, lo, tri_mode, sA,
                                             sB, sC, kchunk);
  GPGP_CHECK_LAUNCH();
}

static void gemm64_dispatch(cudaStream_t s, bool ta, bool tb, dim3 grid, int64_t M, int64_t N, int64_t K,
                            double alpha, const double *A, int64_t lda, const double *B, int64_t ldb,
                            double beta, double *C, int64_t ldc, int lo, int tri_mode, int64_t sA, int64_t sB,
                            int64_t sC, int64_t kchunk) {
  if (!ta && !tb)
    launch_gemm64<false, false>(s, grid, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, lo, tri_mode, sA, sB, sC, kchunk);
  else if (!ta && tb)
    launch_gemm64<false, true>(s, grid, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, lo, tri_mode, sA, sB, sC, kchunk);
  else if (ta && !tb)
    launch_gemm64<true, false>(s, grid, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, lo, tri_mode, sA, sB, sC, kchunk);
  else
    launch_gemm64<true, true>(s, grid, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, lo, tri_mode, sA, sB, sC, kchunk);
}

// Small products (few 64 x 64 tiles, short K): one thread per element of C, so
// that the FP64 work spreads over many SMs instead of a few tile CTAs (an FP64
// warp instruction holds its sub-partition for 64 cycles on this part).
__global__ void gemm64_small_kernel(int64_t M, int64_t N, int64_t K, double alpha, const double *__restrict__ A,
                                    int64_t lda, int ta, const double *__restrict__ B, int64_t ldb, int tb,
                                    double beta, double *__restrict__ C, int64_t ldc, int lower) {
  const int64_t i = (int64_t)blockIdx.x * 32 + (threadIdx.x & 31);
  const int64_t j = (int64_t)blockIdx.y * 8 + (threadIdx.x >> 5);
  if (i >= M || j >= N || (lower && j > i)) return;
  double s0 = 0.0, s1 = 0.0;
  int64_t k = 0;
  for (; k + 1 < K; k += 2) {
    const double a0 = ta ? A[k + i * lda] : A[i + k * lda];
    const double a1 = ta ? A[k + 1 + i * lda] : A[i + (k + 1) * lda];
    const double b0 = tb ? B[j + k * ldb] : B[k + j * ldb];
    const double b1 = tb ? B[j + (k + 1) * ldb] : B[k + 1 + j * ldb];
    s0 = fma(a0, b0, s0);
    s1 = fma(a1, b1, s1);
  }
  if (k < K) s0 = fma(ta ? A[k + i * lda] : A[i + k * lda], tb ? B[j + k * ldb] : B[k + j * ldb], s0);
  const double v = alpha * (s0 + s1);
  C[i + j * ldc] = (beta == 0.0) ? v : v + beta * C[i + j * ldc];
}

void gemm64_batched(cudaStream_t s, bool ta, bool tb, int64_t M, int64_t N, int64_t K, double alpha,
                    const double *A, int64_t lda, int64_t sA, const double *B, int64_t ldb, int64_t sB,
                    double beta, double *C, int64_t ldc, int64_t sC, int64_t batch, bool lower_only,
                    int tri_mode) {
  if (M <= 0 || N <= 0 || batch <= 0) return;
  dim3 grid((unsigned)((M + GBM - 1) / GBM), (unsigned)((N + GBN - 1) / GBN), (unsigned)batch);
  int lo = lower_only ? 1 : 0;
  const int64_t tiles = (int64_t)grid.x * grid.y;
  // few output tiles and a long K (Gram matrices of tall n x M factors): split K
  // over the third grid axis so that every SM gets work, then reduce the
  // partials in a fixed order
  if (batch == 1 && tiles < 152 && K >= 4096) {
    int64_t nz = std::min<int64_t>((2 * 152 + tiles - 1) / tiles, K / 1024);
    const int64_t kchunk = ((K + nz - 1) / nz + GBK - 1) / GBK * GBK;
    nz = (K + kchunk - 1) / kchunk;
    double *P = nullptr;
    GPGP_CUDA(cudaMallocAsync((void **)&P, (size_t)nz * M * N * sizeof(double), s));
    dim3 g2(grid.x, grid.y, (unsigned)nz);
    gemm64_dispatch(s, ta, tb, g2, M, N, K, 1.0, A, lda, B, ldb, 0.0, P, M, 0, tri_mode, 0, 0, M * N, kchunk);
    const int64_t MN = M * N;
    splitk_reduce_kernel<<<(unsigned)std::min<int64_t>((MN + 255) / 256, 4096), 256, 0, s>>>(
        M, N, (int)nz, P, alpha, beta, C, ldc, lo);
    GPGP_CHECK_LAUNCH();
    GPGP_CUDA(cudaFreeAsync(P, s));
    return;
  }
  gemm64_dispatch(s, ta, tb, grid, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, lo, tri_mode, sA, sB, sC, 0);
}

void gemm64(cudaStream_t s, bool ta, bool tb, int64_t M, int64_t N, int64_t K, double alpha,
            const double *A, int64_t lda, const double *B, int64_t ldb, double beta, double *C,
            int64_t ldc, bool lower_only, int tri_mode) {
  // (the batched entry keeps the tile kernel for every batch size, so that a
  // problem's result does not depend on how many others share its launch)
  if (M > 0 && N > 0 && tri_mode == 0 && K <= 256 && ((M + GBM - 1) / GBM) * ((N + GBN - 1) / GBN) < 152) {
    dim3 g((unsigned)((M + 31) / 32), (unsigned)((N + 7) / 8));
    gemm64_small_kernel<<<g, 256, 0, s>>>(M, N, K, alpha, A, lda, ta ? 1 : 0, B, ldb, tb ? 1 : 0, beta, C, ldc,
                                          lower_only ? 1 : 0);
    GPGP_CHECK_LAUNCH();
    return;
  }
  gemm64_batched(s, ta, tb, M, N, K, alpha, A, lda, 0, B, ldb, 0, beta, C, ldc, 0, 1, lower_only,
                 tri_mode);
}

// ---------------------------------------------------------------------------
// diagonal block: factor + invert in shared memory (one CTA)
// ---------------------------------------------------------------------------
// On this part the FP64 pipe retires about 2 lane operations per clock per SM,
// and a warp instruction occupies it whether 1 or 32 lanes are active, so the
// kernel issues as few FP64 warp instructions as it can, each with all lanes on
// distinct entries, and runs the factor and the inverse in one loop with one
// barrier per column:
//  - factor, right-looking: warp 0 takes the pivots one column ahead (column
//    j+1 gets its update from column j, then its inverse square root,
//    rsqrt_fast) while the update warps apply the rank-1 update of column j to
//    the trailing triangle c >= j+2. The trailing triangle's entries are
//    numbered by column, last column first, so that step j's entries are the
//    first (kb-2-j)(kb-1-j)/2 of one fixed list. The warps that share warp 0's
//    sub-partition take no update work; the other twelve (three per
//    sub-partition, enough to cover the FP64 latency) share it evenly.
//  - inverse: W = L^-1 = D^-1 V with D = diag(L) and V the unit lower triangular
//    inverse of the column-scaled factor L D^-1:
//      V(i, c) = -sum_{k=c..i-1} (L(i, k) / L(k, k)) V(k, c),  V(c, c) = 1.
//    The k = c term is written by the pivot of column c (V(i, c) starts as
//    -L(i, c) / L(c, c)); the terms k > c are added right-looking, step k adding
//    V(i, k) V(k, c) to every (i > k, c < k) while V(i, k) still holds only its
//    first term. Step k needs column k of L and rows <= k of V final, so it runs
//    beside the factor's step k + 1 in the same loop iteration. Every inverse
//    entry costs one FMA; the row scaling by 1 / L(i, i) happens once, on the
//    way out.
//  - log L_jj summed in a fixed tree order.
// -x by flipping the sign bit (an integer instruction, not an FP64 one)
__device__ __forceinline__ double neg_bits(double x) {
  return __longlong_as_double(__double_as_longlong(x) ^ (long long)0x8000000000000000ull);
}

__device__ __forceinline__ int div_small(int e, int d, int magic) {
  // e / d for e < 4096, 1 <= d <= 64, magic = ceil(2^20 / d): exact on that range
  return (int)(((unsigned)e * (unsigned)magic) >> 20);
}

__global__ void __launch_bounds__(DIAG_THREADS) potrf_diag_kernel(double *__restrict__ A, int kb, int64_t lda,
                                                         double *__restrict__ Winv,
                                                         double *__restrict__ logdet_part,
                                                         int *__restrict__ status, int64_t k0,
                                                         int64_t sA, int64_t sW, int64_t sL) {
  // batched: problem blockIdx.x (strides sA, sW, sL; status has one word per problem)
  A += blockIdx.x * sA;
  Winv += blockIdx.x * sW;
  logdet_part += blockIdx.x * sL;
  status += blockIdx.x;
  __shared__ double S[NB][NB + 1];
  __shared__ double V[NB][NB + 1];
  __shared__ double rdiag[NB];
  __shared__ double lg[NB];
  __shared__ unsigned short pairs[NB * (NB + 1) / 2];  // (r | c << 8), column-major from the last column
  __shared__ int failed;
  if (*(volatile int *)status != 0) return;
  const int tid = threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5;
  for (int idx = tid; idx < NB * NB; idx += DIAG_THREADS) {
    const int r = idx % NB, c = idx / NB;
    // held negated until its column is pivoted (see the update loop)
    S[r][c] = (r < kb && c < kb && r >= c) ? neg_bits(A[r + c * lda]) : 0.0;
    V[r][c] = 0.0;
  }
  // entry e of the kb x kb triangle: u = kb - 1 - c is the largest u with
  // u (u + 1) / 2 <= e; r = c + e - u (u + 1) / 2 (a partial block lists only its
  // own entries)
  for (int e = tid; e < kb * (kb + 1) / 2; e += DIAG_THREADS) {
    int u = (int)((sqrtf(8.0f * (float)e + 1.0f) - 1.0f) * 0.5f);
    while (u * (u + 1) / 2 > e) --u;
    while ((u + 1) * (u + 2) / 2 <= e) ++u;
    const int c = kb - 1 - u, r = c + (e - u * (u + 1) / 2);
    pairs[e] = (unsigned short)(r | (c << 8));
  }
  if (tid == 0) failed = 0;
  __syncthreads();
  // Warp 0 keeps the current scaled column in registers: lane l owns rows l and
  // l + 32, and lreg[u] holds L(l + 32 u, j) once column j is pivoted. Rows below
  // 32 drop out after column 31, so their FP64 work is skipped from then on (a
  // warp instruction costs the same with one lane or 32).
  double lreg[2] = {0.0, 0.0};
  // pivot of column j by warp 0 from t[u] = -S(l + 32 u, j) after all updates:
  // L_jj, the scaled column below it (stored positive, and kept in lreg) and the
  // first term of column j of V
  auto pivot = [&](int j, const double (&t)[2]) {
    const double dj = neg_bits(__shfl_sync(0xffffffffu, j < 32 ? t[0] : t[1], j & 31));
    // not positive (sign bit or zero) or not finite, tested on the bits
    const long long djb = __double_as_longlong(dj);
    if (djb <= 0ll || (djb >> 52) >= 0x7FFll) {
      if (lane == 0) {
        failed = 1;
        atomicCAS(status, 0, (int)(k0 + j + 1));
      }
      return;
    }
    const double rp = rsqrt_fast(dj);
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      if (u == 1 || j < 31) {
        const int r = lane + 32 * u;
        if (r > j && r < kb) {
          const double l = -(t[u] * rp);
          S[r][j] = l;
          V[r][j] = -(l * rp);
          lreg[u] = l;
        }
      }
    }
    if (lane == (j & 31)) {
      S[j][j] = dj * rp;
      rdiag[j] = rp;
    }
  };
  if (warp == 0) {
    double t0[2];
#pragma unroll
    for (int u = 0; u < 2; ++u) t0[u] = (lane + 32 * u < kb) ? S[lane + 32 * u][0] : 0.0;
    pivot(0, t0);
  }
  __syncthreads();
  if (failed) return;
  // update workers: every warp off sub-partition 0 (warps 4, 8, 12 share warp 0's)
  constexpr int NUPD = DIAG_THREADS / 32 - DIAG_THREADS / 128;  // 12 update warps
  const int uw = warp - 1 - (warp >> 2);
  const int ut = uw * 32 + lane;
  for (int j = 0; j < kb; ++j) {
    if (warp == 0) {
      if (j + 1 < kb) {
        // column j + 1 takes its last update, from column j, then its pivot
        const double l = __shfl_sync(0xffffffffu, (j + 1) < 32 ? lreg[0] : lreg[1], (j + 1) & 31);
        double t[2] = {0.0, 0.0};
#pragma unroll
        for (int u = 0; u < 2; ++u) {
          if (u == 1 || j < 31) {
            const int r = lane + 32 * u;
            if (r > j && r < kb) t[u] = fma(lreg[u], l, S[r][j + 1]);
          }
        }
        pivot(j + 1, t);
      }
    } else if ((warp & 3) != 0) {
      // factor step j: entries (r, c), c >= j + 2, of the fixed list; inverse step
      // k = j - 1: entries (i, c), k < i < kb, c < k, row-major by i. Both are
      // dst += a b with a, b >= sign-free operands (the trailing matrix is held
      // negated), so that each entry is exactly one FP64 instruction.
      const int cf = j < kb - 2 ? (kb - 2 - j) * (kb - 1 - j) / 2 : 0;
      const int k = j - 1;
      const int ci = k >= 1 ? (kb - 1 - k) * k : 0;
      const int magic = k >= 1 ? ((1 << 20) + k - 1) / k : 0;
      for (int e = ut; e < cf + ci; e += NUPD * 32) {
        const double *pa, *pb;
        double *dst;
        if (e < cf) {
          const unsigned short pc = pairs[e];
          const int r = pc & 0xFF, c = pc >> 8;
          dst = &S[r][c];
          pa = &S[r][j];
          pb = &S[c][j];
        } else {
          const int e2 = e - cf;
          const int q = div_small(e2, k, magic);
          const int c = e2 - q * k, i = k + 1 + q;
          dst = &V[i][c];
          pa = &V[i][k];
          pb = &V[k][c];
        }
        *dst = fma(*pa, *pb, *dst);
      }
    }
    __syncthreads();
    if (failed) return;
  }
  // write the factor back (lower part of the block)
  for (int idx = tid; idx < kb * kb; idx += DIAG_THREADS) {
    const int r = idx % kb, c = idx / kb;
    if (r >= c) A[r + c * lda] = S[r][c];
  }
  if (tid < NB) lg[tid] = tid < kb ? log(S[tid][tid]) : 0.0;
  __syncthreads();
  // W = D^-1 V
  for (int idx = tid; idx < NB * NB; idx += DIAG_THREADS) {
    const int r = idx % NB, c = idx / NB;
    double wv = 0.0;
    if (r < kb && c <= r) wv = (r == c) ? rdiag[r] : rdiag[r] * V[r][c];
    Winv[r + c * NB] = wv;
  }
  for (int st = NB / 2; st > 0; st >>= 1) {
    if (tid < st) lg[tid] += lg[tid + st];
    __syncthreads();
  }
  if (tid == 0) *logdet_part = lg[0];
}

// panel: L21 = A21 L11^-T by forward substitution, one row per thread (in place).
// Substitution keeps the factorisation backward stable when a diagonal block is
// ill-conditioned (FITC's K_z); the inverse W is used by the solves instead.
__global__ void __launch_bounds__(128) potrf_panel_kernel(double *__restrict__ A21, int64_t m, int kb,
                                                          int64_t lda, const double *__restrict__ L11,
                                                          const int *__restrict__ status, int64_t sA) {
  // batched: problem blockIdx.y (A21 and L11 offset by sA, one status word per problem)
  A21 += blockIdx.y * sA;
  L11 += blockIdx.y * sA;
  status += blockIdx.y;
  __shared__ double Ls[NB][NB + 1];
  __shared__ double rd[NB];
  if (*(volatile const int *)status != 0) return;
  for (int idx = threadIdx.x; idx < NB * NB; idx += blockDim.x) {
    int r = idx % NB, c = idx / NB;
    Ls[r][c] = (r < kb && c < kb && r >= c) ? L11[r + c * lda] : 0.0;
  }
  __syncthreads();
  if (threadIdx.x < kb) rd[threadIdx.x] = 1.0 / Ls[threadIdx.x][threadIdx.x];
  __syncthreads();
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= m) return;
  double x[NB];
#pragma unroll
  for (int c = 0; c < NB; ++c) {
    if (c < kb) {
      double s = A21[r + c * lda];
      for (int k = 0; k < c; ++k) s = fma(-x[k], Ls[c][k], s);
      x[c] = s * rd[c];
    }
  }
#pragma unroll
  for (int c = 0; c < NB; ++c)
    if (c < kb) A21[r + c * lda] = x[c];
}

// panel by the diagonal block's inverse: L21 = A21 W11^T, L21(r, c) = sum_{k <= c}
// A21(r, k) W11(c, k). A CTA takes 4 rows (one element per thread), staged in
// shared memory with W11, so the FP64 work spreads over m / 4 CTAs. For the
// well-conditioned diagonal blocks of B = I + S K S the error is that of the
// substitution to within the block's condition number.
__global__ void __launch_bounds__(256) potrf_panel_inv_kernel(double *__restrict__ A21, int64_t m, int kb,
                                                              int64_t lda, const double *__restrict__ W,
                                                              const int *__restrict__ status) {
  __shared__ double Ws[NB][NB + 1];
  __shared__ double As[4][NB + 1];
  if (*(volatile const int *)status != 0) return;
  const int64_t r0 = (int64_t)blockIdx.x * 4;
  for (int idx = threadIdx.x; idx < NB * NB; idx += 256) Ws[idx % NB][idx / NB] = W[idx];
  {
    const int rr = threadIdx.x & 3, c = threadIdx.x >> 2;
    As[rr][c] = (r0 + rr < m && c < kb) ? A21[r0 + rr + c * lda] : 0.0;
  }
  __syncthreads();
  const int rr = threadIdx.x & 3, c = threadIdx.x >> 2;
  if (r0 + rr >= m || c >= kb) return;
  double s0 = 0.0, s1 = 0.0;
  int k = 0;
  for (; k + 1 <= c; k += 2) {
    s0 = fma(As[rr][k], Ws[c][k], s0);
    s1 = fma(As[rr][k + 1], Ws[c][k + 1], s1);
  }
  if (k <= c) s0 = fma(As[rr][k], Ws[c][k], s0);
  A21[r0 + rr + c * lda] = s0 + s1;
}

void potrf(cudaStream_t s, double *A, int64_t n, int64_t lda, double *Winv, double *logdet_part,
           int *status, int panel_mode) {
  for (int64_t k0 = 0, blk = 0; k0 < n; k0 += NB, ++blk) {
    const int kb = (int)std::min<int64_t>(NB, n - k0);
    double *Akk = A + k0 + k0 * lda;
    double *W = Winv + blk * NB * NB;
    {
      KTScope kts(GPGP_KPROF_POTRF_DIAG, s, 2.0 * kb * kb * kb / 3);
      potrf_diag_kernel<<<1, DIAG_THREADS, 0, s>>>(Akk, kb, lda, W, logdet_part + blk, status, k0, 0, 0, 0);
    }
    GPGP_CHECK_LAUNCH();
    const int64_t m = n - k0 - kb;
    if (m > 0) {
      double *A21 = A + (k0 + kb) + k0 * lda;
      if (panel_mode == 1)
        potrf_panel_inv_kernel<<<(unsigned)((m + 3) / 4), 256, 0, s>>>(A21, m, kb, lda, W, status);
      else
        potrf_panel_kernel<<<(unsigned)((m + 127) / 128), 128, 0, s>>>(A21, m, kb, lda, Akk, status, 0);
      GPGP_CHECK_LAUNCH();
      double *A22 = A + (k0 + kb) + (k0 + kb) * lda;
      gemm64(s, false, true, m, m, kb, -1.0, A21, lda, A21, lda, 1.0, A22, lda, true, 0);
    }
  }
}

// Batched: `batch` problems of the same size n, matrices sA apart, inverses sW
// apart, logdet partials sL apart, one status word each.
void potrf_batched(cudaStream_t s, double *A, int64_t n, int64_t lda, int64_t sA, double *Winv,
                   int64_t sW, double *logdet_part, int64_t sL, int *status, int64_t batch) {
  for (int64_t k0 = 0, blk = 0; k0 < n; k0 += NB, ++blk) {
    const int kb = (int)std::min<int64_t>(NB, n - k0);
    double *Akk = A + k0 + k0 * lda;
    {
      KTScope kts(GPGP_KPROF_POTRF_DIAG, s, 2.0 * kb * kb * kb / 3 * (double)batch);
      potrf_diag_kernel<<<(unsigned)batch, DIAG_THREADS, 0, s>>>(Akk, kb, lda, Winv + blk * NB * NB, logdet_part + blk,
                                                        status, k0, sA, sW, sL);
    }
    GPGP_CHECK_LAUNCH();
    const int64_t m = n - k0 - kb;
    if (m > 0) {
      double *A21 = A + (k0 + kb) + k0 * lda;
      dim3 pg((unsigned)((m + 127) / 128), (unsigned)batch);
      potrf_panel_kernel<<<pg, 128, 0, s>>>(A21, m, kb, lda, Akk, status, sA);
      GPGP_CHECK_LAUNCH();
      double *A22 = A + (k0 + kb) + (k0 + kb) * lda;
      gemm64_batched(s, false, true, m, m, kb, -1.0, A21, lda, sA, A21, lda, sA, 1.0, A22, lda, sA, batch,
                     true, 0);
    }
  }
}

// ---------------------------------------------------------------------------
// triangular solves with one right-hand side
// ---------------------------------------------------------------------------
// Step k of the forward solve: every CTA recomputes xk = W_kk b_k (64x64), CTA 0
// stores it into xo, and each CTA updates its 256-row slice of b below the block.
__global__ void __launch_bounds__(256) trsv_fwd_step(const double *__restrict__ L, int64_t n, int64_t lda,
                                                     const double *__restrict__ W, int64_t k0, int kb,
                                                     double *__restrict__ b, double *__restrict__ xo,
                                                     const int *__restrict__ status) {
  __shared__ double bk[NB];
  __shared__ double xk[NB];
  if (*(volatile const int *)status != 0) return;
  const int tid = threadIdx.x;
  if (tid < NB) bk[tid] = tid < kb ? b[k0 + tid] : 0.0;
  __syncthreads();
  if (tid < NB) {
    double s = 0.0;
    for (int c = 0; c <= tid && c < kb; ++c) s = fma(W[tid + c * NB], bk[c], s);
    xk[tid] = tid < kb ? s : 0.0;
  }
  __syncthreads();
  if (blockIdx.x == 0 && tid < kb) xo[k0 + tid] = xk[tid];
  const int64_t r = k0 + kb + (int64_t)blockIdx.x * 256 + tid;
  if (r < n) {
    double s = 0.0;
    for (int c = 0; c < kb; ++c) s = fma(L[r + (k0 + c) * lda], xk[c], s);
    b[r] -= s;
  }
}

void trsv_lower(cudaStream_t s, const double *L, int64_t n, int64_t lda, const double *Winv,
                double *b, double *x, const int *status) {
  // b is consumed (rows below the current block are updated in place); x receives L^-1 b
  for (int64_t k0 = 0, blk = 0; k0 < n; k0 += NB, ++blk) {
    const int kb = (int)std::min<int64_t>(NB, n - k0);
    const int64_t rest = n - k0 - kb;
    unsigned g = (unsigned)std::max<int64_t>(1, (rest + 255) / 256);
    trsv_fwd_step<<<g, 256, 0, s>>>(L, n, lda, Winv + blk * NB * NB, k0, kb, b, x, status);
    GPGP_CHECK_LAUNCH();
  }
}

// Backward step: x_k = W_kk^T b_k, then b[0:k0] -= L[k-block rows, 0:k0]^T x_k.
__global__ void __launch_bounds__(256) trsv_bwd_step(const double *__restrict__ L, int64_t lda,
                                                     const double *__restrict__ W, int64_t k0, int kb,
                                                     double *__restrict__ b, double *__restrict__ xo,
                                                     const int *__restrict__ status) {
  __shared__ double bk[NB];
  __shared__ double xk[NB];
  if (*(volatile const int *)status != 0) return;
  const int tid = threadIdx.x;
  if (tid < NB) bk[tid] = tid < kb ? b[k0 + tid] : 0.0;
  __syncthreads();
  if (tid < NB) {
    double s = 0.0;
    for (int r = tid; r < kb; ++r) s = fma(W[r + tid * NB], bk[r], s);
    xk[tid] = tid < kb ? s : 0.0;
  }
  __syncthreads();
  if (blockIdx.x == 0 && tid < kb) xo[k0 + tid] = xk[tid];
  // one warp per column c < k0
  const int lane = tid & 31, warp = tid >> 5;
  const int64_t c = (int64_t)blockIdx.x * 8 + warp;
  if (c < k0) {
    double s = 0.0;
    for (int r = lane; r < kb; r += 32) s = fma(L[(k0 + r) + c * lda], xk[r], s);
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) b[c] -= s;
  }
}

void trsv_lower_t(cudaStream_t s, const double *L, int64_t n, int64_t lda, const double *Winv,
                  double *b, double *x, const int *status) {
  // b is consumed; x receives L^-T b
  const int64_t nblk = (n + NB - 1) / NB;
  for (int64_t blk = nblk - 1; blk >= 0; --blk) {
    const int64_t k0 = blk * NB;
    const int kb = (int)std::min<int64_t>(NB, n - k0);
    unsigned g = (unsigned)std::max<int64_t>(1, (k0 + 7) / 8);
    trsv_bwd_step<<<g, 256, 0, s>>>(L, lda, Winv + blk * NB * NB, k0, kb, b, x, status);
    GPGP_CHECK_LAUNCH();
  }
}

// ---------------------------------------------------------------------------
// single-launch triangular solves, ordered by per-block flags
// ---------------------------------------------------------------------------
// A persistent grid takes the 64-row blocks of x in dependency order from a
// ticket (forward: first block first; transposed: last block first), so every
// block a CTA waits for belongs to a CTA that is already running. The CTA of
// block i subtracts L_ij x_j (L_ji^T x_j when transposed) for each earlier block
// j as soon as that block's flag is set, then multiplies by the diagonal block's
// inverse W_ii, writes x_i and sets its flag. Each thread visits the blocks in a
// fixed order, so the result does not depend on timing. Waits are bounded: when
// one runs out the kernel sets *err = 3 and every CTA leaves.
// sync: [0] ticket, [1 + blk] done flag of block blk; zeroed before the launch.
constexpr int FLOW_BATCH = 8;  // earlier blocks applied per round

__global__ void __launch_bounds__(256) trsv_flow_kernel(const double *__restrict__ L, int64_t n, int64_t lda,
                                                        const double *__restrict__ Winv,
                                                        const double *__restrict__ b, double *x, int trans,
                                                        const int *__restrict__ status, unsigned *sync,
                                                        int *err) {
  __shared__ double Ws[NB][NB + 1];
  __shared__ double xs[FLOW_BATCH][NB];
  __shared__ double vs[NB];
  __shared__ double red[4][NB + 1];
  __shared__ int64_t step_sh;
  __shared__ int k_sh;
  if (*(volatile const int *)status != 0) return;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t nblk = (n + NB - 1) / NB;
  volatile unsigned *done = sync + 1;
  for (;;) {
    __syncthreads();
    if (tid == 0) step_sh = (int64_t)atomicAdd(sync, 1u);
    __syncthreads();
    const int64_t step = step_sh;
    if (step >= nblk) return;
    const int64_t blk = trans ? nblk - 1 - step : step;
    const int64_t k0 = blk * NB;
    const int kb = (int)((n - k0) < NB ? (n - k0) : NB);
    const double *W = Winv + blk * NB * NB;
    for (int idx = tid; idx < NB * NB; idx += 256) Ws[idx % NB][idx / NB] = W[idx];
    // forward: thread (r, p) takes row r of the block and columns 16p..16p+15 of
    // every earlier block; transposed: warp w takes columns 8w..8w+7 of this block
    // and lane l rows l, l + 32 of every later block
    double acc[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) acc[q] = 0.0;
    const int r = tid & 63, p = tid >> 6;
    const int64_t ndep = trans ? nblk - 1 - blk : blk;
    // This thread's 16 entries of the L tile of earlier block number d; the tile of
    // the next block is always in flight (loaded before the wait for its flag and
    // before the products with the current one).
    auto load_tile = [&](int64_t d, double (&t)[16]) {
      const int64_t j = trans ? nblk - 1 - d : d;
      const int64_t j0 = j * NB;
      const int jb = (int)((n - j0) < NB ? (n - j0) : NB);
      if (!trans) {
        const double *Lr = L + (k0 + r) + (j0 + 16 * p) * lda;
#pragma unroll
        for (int q = 0; q < 16; ++q) t[q] = (r < kb && 16 * p + q < jb) ? Lr[q * lda] : 0.0;
      } else {
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          const int c = warp * 8 + q;
          const double *Lc = L + j0 + (k0 + c) * lda;
          t[2 * q] = (c < kb && lane < jb) ? Lc[lane] : 0.0;
          t[2 * q + 1] = (c < kb && lane + 32 < jb) ? Lc[lane + 32] : 0.0;
        }
      }
    };
    double tnext[16];
    if (ndep > 0) load_tile(0, tnext);
    for (int64_t d0 = 0; d0 < ndep;) {
      // warp 0 finds how many of the next (up to) eight blocks are done
      if (warp == 0) {
        const int avail = (int)((ndep - d0) < FLOW_BATCH ? (ndep - d0) : FLOW_BATCH);
        int k = -1;
        for (uint32_t it = 0; it < (1u << 21); ++it) {
          const int64_t jl = trans ? nblk - 1 - (d0 + lane) : d0 + lane;
          const bool ready = lane < avail && done[jl] != 0u;
          const unsigned m = __ballot_sync(0xffffffffu, ready);
          const int run = __ffs(~m) - 1;  // consecutive done blocks from d0
          if (run > 0) {
            k = run;
            break;
          }
          if ((it & 1023u) == 1023u && *(volatile const int *)err != 0) break;
          __nanosleep(64);
        }
        if (lane == 0) {
          if (k < 0) atomicExch(err, 3);
          k_sh = k;
        }
      }
      __syncthreads();
      const int k = k_sh;
      if (k < 0) return;
      __threadfence();
      for (int idx = tid; idx < k * NB; idx += 256) {
        const int dd = idx / NB, c = idx % NB;
        const int64_t j = trans ? nblk - 1 - (d0 + dd) : d0 + dd;
        xs[dd][c] = j * NB + c < n ? __ldcg(x + j * NB + c) : 0.0;
      }
      __syncthreads();
      for (int dd = 0; dd < k; ++dd) {
        double tc[16];
#pragma unroll
        for (int q = 0; q < 16; ++q) tc[q] = tnext[q];
        if (d0 + dd + 1 < ndep) load_tile(d0 + dd + 1, tnext);
        if (!trans) {
#pragma unroll
          for (int q = 0; q < 16; ++q) acc[q & 7] = fma(tc[q], xs[dd][16 * p + q], acc[q & 7]);
        } else {
#pragma unroll
          for (int q = 0; q < 8; ++q) acc[q] += fma(tc[2 * q + 1], xs[dd][lane + 32], tc[2 * q] * xs[dd][lane]);
        }
      }
      __syncthreads();
      d0 += k;
    }
    // v = b_blk - (the sum over the earlier blocks)
    if (!trans) {
      double t = 0.0;
#pragma unroll
      for (int q = 0; q < 8; ++q) t += acc[q];
      red[p][r] = t;
      __syncthreads();
      if (tid < NB) vs[tid] = tid < kb ? b[k0 + tid] - (((red[0][tid] + red[1][tid]) + red[2][tid]) + red[3][tid]) : 0.0;
    } else {
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        double t = acc[q];
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        acc[q] = t;
      }
      if (lane < 8) {
        const int c = warp * 8 + lane;
        double t = acc[0];
#pragma unroll
        for (int q = 1; q < 8; ++q) t = lane == q ? acc[q] : t;
        vs[c] = c < kb ? b[k0 + c] - t : 0.0;
      }
    }
    __syncthreads();
    // x_blk = W v (lower W) or W^T v: four threads per entry, partial sums by shuffles
    {
      const int row = tid >> 2, pp = tid & 3;
      double s0 = 0.0, s1 = 0.0;
      if (!trans) {
        for (int c = pp; c <= row && c < kb; c += 8) {
          s0 = fma(Ws[row][c], vs[c], s0);
          if (c + 4 <= row && c + 4 < kb) s1 = fma(Ws[row][c + 4], vs[c + 4], s1);
        }
      } else {
        for (int rr = row + pp; rr < kb; rr += 8) {
          s0 = fma(Ws[rr][row], vs[rr], s0);
          if (rr + 4 < kb) s1 = fma(Ws[rr + 4][row], vs[rr + 4], s1);
        }
      }
      double s = s0 + s1;
      s += __shfl_xor_sync(0xffffffffu, s, 1);
      s += __shfl_xor_sync(0xffffffffu, s, 2);
      if (pp == 0 && row < kb) {
        x[k0 + row] = s;
        __threadfence();
      }
    }
    __syncthreads();
    if (tid == 0) {
      __threadfence();
      atomicExch((unsigned *)(done + blk), 1u);
    }
  }
}

// Small solves (n <= 512): one CTA walks the row blocks in order (a launch and a
// 64-row step cost less than the flags of the multi-CTA version at this size).
// Thread (r, p) sums the earlier (later, when transposed) blocks' columns
// c = p mod 4 for row r of the block; the block's inverse then gives x_blk.
__global__ void __launch_bounds__(256) trsv_small_kernel(const double *__restrict__ L, int64_t n, int64_t lda,
                                                         const double *__restrict__ Winv,
                                                         const double *__restrict__ b, double *__restrict__ x,
                                                         int trans, const int *__restrict__ status) {
  __shared__ double xs[8 * NB];
  __shared__ double vs[NB];
  __shared__ double red[4][NB + 1];
  if (*(volatile const int *)status != 0) return;
  const int tid = threadIdx.x, r = tid & 63, p = tid >> 6;
  const int nblk = (int)((n + NB - 1) / NB);
  for (int st = 0; st < nblk; ++st) {
    const int blk = trans ? nblk - 1 - st : st;
    const int k0 = blk * NB;
    const int kb = (int)(n - k0 < NB ? n - k0 : NB);
    double acc = 0.0;
    if (r < kb) {
      if (!trans)
        for (int c = p; c < k0; c += 4) acc = fma(L[(k0 + r) + (int64_t)c * lda], xs[c], acc);
      else
        for (int c = k0 + kb + p; c < n; c += 4) acc = fma(L[c + (int64_t)(k0 + r) * lda], xs[c], acc);
    }
    red[p][r] = acc;
    __syncthreads();
    if (tid < NB) vs[tid] = tid < kb ? b[k0 + tid] - (((red[0][tid] + red[1][tid]) + red[2][tid]) + red[3][tid]) : 0.0;
    __syncthreads();
    if (tid < kb) {
      const double *W = Winv + (int64_t)blk * NB * NB;
      double s0 = 0.0, s1 = 0.0;
      if (!trans) {
        int c = 0;
        for (; c + 1 <= tid; c += 2) {
          s0 = fma(W[tid + c * NB], vs[c], s0);
          s1 = fma(W[tid + (c + 1) * NB], vs[c + 1], s1);
        }
        if (c <= tid) s0 = fma(W[tid + c * NB], vs[c], s0);
      } else {
        int rr = tid;
        for (; rr + 1 < kb; rr += 2) {
          s0 = fma(W[rr + tid * NB], vs[rr], s0);
          s1 = fma(W[rr + 1 + tid * NB], vs[rr + 1], s1);
        }
        if (rr < kb) s0 = fma(W[rr + tid * NB], vs[rr], s0);
      }
      xs[k0 + tid] = s0 + s1;
      x[k0 + tid] = s0 + s1;
    }
    __syncthreads();
  }
}

void trsv_flow(cudaStream_t s, const double *L, int64_t n, int64_t lda, const double *Winv, const double *b,
               double *x, bool trans, const int *status, unsigned *sync, int *err) {
  if (n <= 0) return;
  const int g_sms = device_sms();
  const int64_t nblk = (n + NB - 1) / NB;
  if (nblk <= 8) {
    KTScope kts(GPGP_KPROF_TRSV, s, (double)n * (double)n);
    trsv_small_kernel<<<1, 256, 0, s>>>(L, n, lda, Winv, b, x, trans ? 1 : 0, status);
    GPGP_CHECK_LAUNCH();
    return;
  }
  GPGP_CUDA(cudaMemsetAsync(sync, 0, (size_t)(nblk + 1) * sizeof(unsigned), s));
  const unsigned grid = (unsigned)std::min<int64_t>(nblk, g_sms);
  KTScope kts(GPGP_KPROF_TRSV, s, (double)n * (double)n);
  trsv_flow_kernel<<<grid, 256, 0, s>>>(L, n, lda, Winv, b, x, trans ? 1 : 0, status, sync, err);
  GPGP_CHECK_LAUNCH();
}

// ---------------------------------------------------------------------------
// substitution solves for small factors (M x M lower L), as R's forwardsolve /
// backsolve do: rows of a column-major n x M matrix, one thread per row
// ---------------------------------------------------------------------------
// mode 0: X = B L^-T (x L^T = b, forward); mode 1: X = B L^-1 (x L = b, backward).
// X may alias B.
__global__ void tri_rows_kernel(const double *__restrict__ L, int64_t M, int64_t ldl, const double *B,
                                int64_t ldb, double *X, int64_t ldx, int64_t n, int mode) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (mode == 0) {
    for (int64_t c = 0; c < M; ++c) {
      double s = B[i + c * ldb];
      for (int64_t k = 0; k < c; ++k) s = fma(-X[i + k * ldx], L[c + k * ldl], s);
      X[i + c * ldx] = s / L[c + c * ldl];
    }
  } else {
    for (int64_t c = M - 1; c >= 0; --c) {
      double s = B[i + c * ldb];
      for (int64_t k = c + 1; k < M; ++k) s = fma(-X[i + k * ldx], L[k + c * ldl], s);
      X[i + c * ldx] = s / L[c + c * ldl];
    }
  }
}

void tri_rows(cudaStream_t s, const double *L, int64_t M, int64_t ldl, const double *B, int64_t ldb,
              double *X, int64_t ldx, int64_t n, int mode) {
  if (n <= 0 || M <= 0) return;
  tri_rows_kernel<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(L, M, ldl, B, ldb, X, ldx, n, mode);
  GPGP_CHECK_LAUNCH();
}

// one warp: x = L^-1 b (trans = 0) or x = L^-T b (trans = 1), x may alias b
__global__ void tri_vec_kernel(const double *__restrict__ L, int64_t M, int64_t ldl, const double *b,
                               double *x, int trans) {
  const int lane = threadIdx.x & 31;
  if (!trans) {
    for (int64_t r = 0; r < M; ++r) {
      double s = 0.0;
      for (int64_t k = lane; k < r; k += 32) s = fma(L[r + k * ldl], x[k], s);
      for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      if (lane == 0) x[r] = (b[r] - s) / L[r + r * ldl];
      __syncwarp();
    }
  } else {
    for (int64_t r = M - 1; r >= 0; --r) {
      double s = 0.0;
      for (int64_t k = r + 1 + lane; k < M; k += 32) s = fma(L[k + r * ldl], x[k], s);
      for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      if (lane == 0) x[r] = (b[r] - s) / L[r + r * ldl];
      __syncwarp();
    }
  }
}

void tri_vec(cudaStream_t s, const double *L, int64_t M, int64_t ldl, const double *b, double *x,
             bool trans) {
  if (M <= 0) return;
  tri_vec_kernel<<<1, 32, 0, s>>>(L, M, ldl, b, x, trans ? 1 : 0);
  GPGP_CHECK_LAUNCH();
}

// ---------------------------------------------------------------------------
// multi-RHS solve and triangular inverse
// ---------------------------------------------------------------------------
void trsm_lower(cudaStream_t s, const double *L, int64_t n, int64_t lda, const double *Winv,
                double *B, int64_t m, int64_t ldb, double *tmp, const int *status) {
  // right-looking: X_k = W_kk B_k; B_rest -= L_rest,k X_k. tmp holds NB x m.
  (void)status;
  for (int64_t k0 = 0, blk = 0; k0 < n; k0 += NB, ++blk) {
    const int kb = (int)std::min<int64_t>(NB, n - k0);
    double *Bk = B + k0;
    gemm64(s, false, false, kb, m, kb, 1.0, Winv + blk * NB * NB, NB, Bk, ldb, 0.0, tmp, NB);
    GPGP_CUDA(cudaMemcpy2DAsync(Bk, ldb * sizeof(double), tmp, NB * sizeof(double),
                                kb * sizeof(double), m, cudaMemcpyDeviceToDevice, s));
    const int64_t rest = n - k0 - kb;
    if (rest > 0)
      gemm64(s, false, false, rest, m, kb, -1.0, L + (k0 + kb) + k0 * lda, lda, tmp, NB, 1.0,
             B + k0 + kb, ldb);
  }
}

__global__ void set_identity_kernel(double *W, int64_t n, int64_t ldw) {
  for (int64_t j = blockIdx.y; j < n; j += gridDim.y)
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
      W[i + j * ldw] = (i == j) ? 1.0 : 0.0;
}

void trtri_lower(cudaStream_t s, const double *L, int64_t n, int64_t lda, const double *Winv,
                 double *Wout, int64_t ldw, double *tmp, const int *status) {
  // Wout = L^-1 by a triangular solve against I that skips the zero columns:
  // for block row k, X_k = W_kk B_k[:, 0:k0+kb] and B_rest[:, 0:k0+kb] -= L_rest,k X_k.
  // tmp holds NB x n. The strict upper triangle of Wout stays exactly zero.
  (void)status;
  if (n == 0) return;
  dim3 g((unsigned)std::min<int64_t>((n + 255) / 256, 64), (unsigned)std::min<int64_t>(n, 65535));
  set_identity_kernel<<<g, 256, 0, s>>>(Wout, n, ldw);
  GPGP_CHECK_LAUNCH();
  for (int64_t k0 = 0, blk = 0; k0 < n; k0 += NB, ++blk) {
    const int kb = (int)std::min<int64_t>(NB, n - k0);
    const int64_t ncol = k0 + kb;
    double *Bk = Wout + k0;
    gemm64(s, false, false, kb, ncol, kb, 1.0, Winv + blk * NB * NB, NB, Bk, ldw, 0.0, tmp, NB);
    GPGP_CUDA(cudaMemcpy2DAsync(Bk, ldw * sizeof(double), tmp, NB * sizeof(double),
                                kb * sizeof(double), ncol, cudaMemcpyDeviceToDevice, s));
    const int64_t rest = n - ncol;
    if (rest > 0)
      gemm64(s, false, false, rest, ncol, kb, -1.0, L + ncol + k0 * lda, lda, tmp, NB, 1.0,
             Wout + ncol, ldw);
  }
}

// column sums of squares of a lower-triangular W (diag of W^T W)
__global__ void col_sumsq_lower_kernel(const double *__restrict__ W, int64_t n, int64_t ldw,
                                       double *__restrict__ out) {
  const int lane = threadIdx.x & 31;
  const int64_t c = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (c >= n) return;
  double s = 0.0;
  for (int64_t r = c + lane; r < n; r += 32) {
    double v = W[r + c * ldw];
    s = fma(v, v, s);
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if (lane == 0) out[c] = s;
}

void col_sumsq_lower(cudaStream_t s, const double *W, int64_t n, int64_t ldw, double *out) {
  if (n == 0) return;
  col_sumsq_lower_kernel<<<(unsigned)((n * 32 + 255) / 256), 256, 0, s>>>(W, n, ldw, out);
  GPGP_CHECK_LAUNCH();
}

__global__ void col_sumsq_kernel(const double *__restrict__ B, int64_t n, int64_t m, int64_t ldb,
                                 double *__restrict__ out) {
  const int lane = threadIdx.x & 31;
  const int64_t c = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (c >= m) return;
  double s = 0.0;
  for (int64_t r = lane; r < n; r += 32) {
    double v = B[r + c * ldb];
    s = fma(v, v, s);
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if (lane == 0) out[c] = s;
}

void col_sumsq(cudaStream_t s, const double *B, int64_t n, int64_t m, int64_t ldb, double *out) {
  if (m == 0) return;
  col_sumsq_kernel<<<(unsigned)((m * 32 + 255) / 256), 256, 0, s>>>(B, n, m, ldb, out);
  GPGP_CHECK_LAUNCH();
}

// ---------------------------------------------------------------------------
// GEMV with a deterministic two-stage reduction over column chunks
// ---------------------------------------------------------------------------
constexpr int GV_ROWS = 256, GV_COLS = 1024;

__global__ void gemv_n_kernel(int64_t M, int64_t N, const double *__restrict__ A, int64_t lda,
                              const double *__restrict__ x, double *__restrict__ part) {
  const int64_t r = (int64_t)blockIdx.x * GV_ROWS + threadIdx.x;
  const int64_t c0 = (int64_t)blockIdx.y * GV_COLS;
  const int64_t c1 = (c0 + GV_COLS < N) ? c0 + GV_COLS : N;
  if (r >= M) return;
  double s = 0.0;
  for (int64_t c = c0; c < c1; ++c) s = fma(A[r + c * lda], x[c], s);
  part[r + blockIdx.y * M] = s;
}

__global__ void gemv_t_kernel(int64_t M, int64_t N, const double *__restrict__ A, int64_t lda,
                              const double *__restrict__ x, double *__restrict__ y, double alpha,
                              double beta) {
  // y[c] = alpha * sum_r A[r, c] x[r] + beta y[c]; one warp per column
  const int lane = threadIdx.x & 31;
  const int64_t c = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (c >= N) return;
  double s = 0.0;
  for (int64_t r = lane; r < M; r += 32) s = fma(A[r + c * lda], x[r], s);
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if (lane == 0) y[c] = (beta == 0.0) ? alpha * s : alpha * s + beta * y[c];
}

__global__ void gemv_reduce_kernel(int64_t M, int nchunk, const double *__restrict__ part,
                                   double alpha, double beta, double *__restrict__ y) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= M) return;
  double s = 0.0;
  for (int k = 0; k < nchunk; ++k) s += part[r + k * M];
  y[r] = (beta == 0.0) ? alpha * s : alpha * s + beta * y[r];
}

// Lower-triangular W (n x n, strict upper zero): y = W x (column chunks above a row
// block are skipped) or y = W^T x (a column's warp starts at its diagonal's
// 32-row group). Half the FP64 work of a full gemv, which bounds it on this part.
__global__ void trmv_n_kernel(int64_t n, const double *__restrict__ W, int64_t ldw, const double *__restrict__ x,
                              double *__restrict__ part) {
  const int64_t r = (int64_t)blockIdx.x * GV_ROWS + threadIdx.x;
  const int64_t c0 = (int64_t)blockIdx.y * GV_COLS;
  const int64_t rmax = (int64_t)blockIdx.x * GV_ROWS + GV_ROWS;  // columns >= rmax are zero for this block
  int64_t c1 = (c0 + GV_COLS < n) ? c0 + GV_COLS : n;
  if (c1 > rmax) c1 = rmax;
  if (r >= n) return;
  double s = 0.0;
  for (int64_t c = c0; c < c1; ++c) s = fma(W[r + c * ldw], x[c], s);
  part[r + blockIdx.y * n] = s;
}

__global__ void trmv_t_kernel(int64_t n, const double *__restrict__ W, int64_t ldw, const double *__restrict__ x,
                              double *__restrict__ y) {
  const int lane = threadIdx.x & 31;
  const int64_t c = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (c >= n) return;
  double s = 0.0;
  for (int64_t r = (c & ~(int64_t)31) + lane; r < n; r += 32) s = fma(W[r + c * ldw], x[r], s);
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if (lane == 0) y[c] = s;
}

void trmv_lower(cudaStream_t s, bool trans, int64_t n, const double *W, int64_t ldw, const double *x, double *y) {
  if (n <= 0) return;
  if (trans) {
    trmv_t_kernel<<<(unsigned)((n * 32 + 255) / 256), 256, 0, s>>>(n, W, ldw, x, y);
    GPGP_CHECK_LAUNCH();
    return;
  }
  const int nchunk = (int)std::max<int64_t>(1, (n + GV_COLS - 1) / GV_COLS);
  double *part = nullptr;
  GPGP_CUDA(cudaMallocAsync((void **)&part, (size_t)n * nchunk * sizeof(double), s));
  dim3 grid((unsigned)((n + GV_ROWS - 1) / GV_ROWS), (unsigned)nchunk);
  trmv_n_kernel<<<grid, GV_ROWS, 0, s>>>(n, W, ldw, x, part);
  GPGP_CHECK_LAUNCH();
  gemv_reduce_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, nchunk, part, 1.0, 0.0, y);
  GPGP_CHECK_LAUNCH();
  GPGP_CUDA(cudaFreeAsync(part, s));
}

void gemv64(cudaStream_t s, bool trans, int64_t M, int64_t N, double alpha, const double *A,
            int64_t lda, const double *x, double beta, double *y) {
  if (trans) {
    if (N == 0) return;
    gemv_t_kernel<<<(unsigned)((N * 32 + 255) / 256), 256, 0, s>>>(M, N, A, lda, x, y, alpha, beta);
    GPGP_CHECK_LAUNCH();
    return;
  }
  if (M == 0) return;
  const int nchunk = (int)std::max<int64_t>(1, (N + GV_COLS - 1) / GV_COLS);
  // partial sums of the column chunks: stream-ordered scratch of this call
  double *part = nullptr;
  GPGP_CUDA(cudaMallocAsync((void **)&part, (size_t)M * nchunk * sizeof(double), s));
  dim3 grid((unsigned)((M + GV_ROWS - 1) / GV_ROWS), (unsigned)nchunk);
  gemv_n_kernel<<<grid, GV_ROWS, 0, s>>>(M, N, A, lda, x, part);
  GPGP_CHECK_LAUNCH();
  gemv_reduce_kernel<<<(unsigned)((M + 255) / 256), 256, 0, s>>>(M, nchunk, part, alpha,
                                                                  beta, y);
  GPGP_CHECK_LAUNCH();
  GPGP_CUDA(cudaFreeAsync(part, s));
}

// ---------------------------------------------------------------------------
// reductions
// ---------------------------------------------------------------------------
__global__ void sum_vec_kernel(const double *__restrict__ v, int64_t n, double *__restrict__ out) {
  __shared__ double red[256];
  double s = 0.0;
  for (int64_t i = threadIdx.x; i < n; i += 256) s += v[i];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int st = 128; st > 0; st >>= 1) {
    if (threadIdx.x < st) red[threadIdx.x] += red[threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[0] = red[0];
}

void sum_vec(cudaStream_t s, const double *v, int64_t n, double *out) {
  sum_vec_kernel<<<1, 256, 0, s>>>(v, n, out);
  GPGP_CHECK_LAUNCH();
}

// ---------------------------------------------------------------------------
// LU with partial pivoting of a small general matrix (the symmetric indefinite
// Schur complement of the bad sites in the non-log-concave fits, where the
// reference takes Matrix::lu of K + diag(V), R/laplace.R:113, R/ep.R:128)
// ---------------------------------------------------------------------------
// Column k: one CTA picks the pivot (largest |A_ik|, i >= k, first index on
// ties), swaps rows k and p across all columns and divides the column below the
// pivot by it; a grid then applies the rank-1 update to the trailing block.
__global__ void __launch_bounds__(256) lu_pivot_kernel(double *__restrict__ A, int64_t n, int64_t lda,
                                                       int64_t k, int *__restrict__ piv,
                                                       int *__restrict__ status) {
  __shared__ double bv[256];
  __shared__ int64_t bi[256];
  if (*(volatile int *)status != 0) return;
  double best = -1.0;
  int64_t arg = k;
  for (int64_t i = k + threadIdx.x; i < n; i += 256) {
    const double v = fabs(A[i + k * lda]);
    if (v > best) {
      best = v;
      arg = i;
    }
  }
  bv[threadIdx.x] = best;
  bi[threadIdx.x] = arg;
  __syncthreads();
  for (int st = 128; st > 0; st >>= 1) {
    if (threadIdx.x < st) {
      const double o = bv[threadIdx.x + st];
      const int64_t oi = bi[threadIdx.x + st];
      if (o > bv[threadIdx.x] || (o == bv[threadIdx.x] && oi < bi[threadIdx.x])) {
        bv[threadIdx.x] = o;
        bi[threadIdx.x] = oi;
      }
    }
    __syncthreads();
  }
  const int64_t p = bi[0];
  if (!(bv[0] > 0.0)) {  // exactly singular (or NaN)
    if (threadIdx.x == 0) atomicCAS(status, 0, (int)(k + 1));
    return;
  }
  if (threadIdx.x == 0) piv[k] = (int)p;
  if (p != k)
    for (int64_t j = threadIdx.x; j < n; j += 256) {
      const double t = A[k + j * lda];
      A[k + j * lda] = A[p + j * lda];
      A[p + j * lda] = t;
    }
  __syncthreads();
  const double r = 1.0 / A[k + k * lda];
  for (int64_t i = k + 1 + threadIdx.x; i < n; i += 256) A[i + k * lda] *= r;
}

__global__ void lu_update_kernel(double *__restrict__ A, int64_t n, int64_t lda, int64_t k,
                                 const int *__restrict__ status) {
  if (*(volatile const int *)status != 0) return;
  const int64_t m = n - k - 1;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < m * m;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = k + 1 + e % m, j = k + 1 + e / m;
    A[i + j * lda] -= A[i + k * lda] * A[k + j * lda];
  }
}

void getrf(cudaStream_t s, double *A, int64_t n, int64_t lda, int *piv, int *status) {
  for (int64_t k = 0; k < n; ++k) {
    lu_pivot_kernel<<<1, 256, 0, s>>>(A, n, lda, k, piv, status);
    GPGP_CHECK_LAUNCH();
    const int64_t m = n - k - 1;
    if (m > 0) {
      const unsigned g = (unsigned)std::min<int64_t>((m * m + 255) / 256, 4 * 152);
      lu_update_kernel<<<g, 256, 0, s>>>(A, n, lda, k, status);
      GPGP_CHECK_LAUNCH();
    }
  }
}

// X <- A^-1 X with the factors of getrf: the row interchanges in order, then the
// unit lower and the upper substitutions. One warp per right-hand side; the
// lanes share each row's dot product.
__global__ void getrs_kernel(const double *__restrict__ LU, int64_t n, int64_t lda, const int *__restrict__ piv,
                             double *__restrict__ X, int64_t m, int64_t ldx, const int *__restrict__ status) {
  const int64_t c = (int64_t)blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  const int lane = threadIdx.x & 31;
  if (c >= m || *(volatile const int *)status != 0) return;
  double *x = X + c * ldx;
  if (lane == 0)
    for (int64_t k = 0; k < n; ++k) {
      const int64_t p = piv[k];
      if (p != k) {
        const double t = x[k];
        x[k] = x[p];
        x[p] = t;
      }
    }
  __syncwarp();
  for (int64_t i = 1; i < n; ++i) {  // unit lower
    double acc = 0.0;
    for (int64_t j = lane; j < i; j += 32) acc = fma(LU[i + j * lda], x[j], acc);
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) x[i] -= acc;
    __syncwarp();
  }
  for (int64_t i = n - 1; i >= 0; --i) {  // upper
    double acc = 0.0;
    for (int64_t j = i + 1 + lane; j < n; j += 32) acc = fma(LU[i + j * lda], x[j], acc);
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) x[i] = (x[i] - acc) / LU[i + i * lda];
    __syncwarp();
  }
}

void getrs(cudaStream_t s, const double *LU, int64_t n, int64_t lda, const int *piv, double *X, int64_t m,
           int64_t ldx, const int *status) {
  if (n <= 0 || m <= 0) return;
  getrs_kernel<<<(unsigned)((m + 7) / 8), 256, 0, s>>>(LU, n, lda, piv, X, m, ldx, status);
  GPGP_CHECK_LAUNCH();
}

}  // namespace gpgp
