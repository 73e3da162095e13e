// Mixed-precision dense kernels: FP64-accurate products on the tcgen05
// tensor cores through exact BF16 slicing (an Ozaki-style split).
//
// Every operand row is scaled by a power of two so that its largest entry is
// in [0.5, 1) and then cut into S 8-bit fixed-point slices (S = 4 or 5)
//   x = 2^e * sum_t q_t 2^-8(t+1),  q_t integers in [-256, 256].
// Slice t is stored as the BF16 value q_t 2^-8t (exact: an 8-bit integer times
// a power of two), so the product of slices t and u already carries its level
// weight 2^-8(t+u) and products of different levels can share an accumulator.
// Levels 0, 1 and 2 get their own FP32 accumulators in TMEM, levels 3.. share
// a fourth: a level-l sum of up to 256 products has 24 significant bits for
// l <= 2, so those sums are exact in FP32; the shared deeper levels round at
// 2^-50 of the result. After every 256-wide K group the four accumulators are
// added into a double-float (hi, lo) pair; at the end of the tile the pair is
// turned into a double with integer instructions and added to C (one FP64 add):
//   (A B^T)_ij = 2^(e_i + f_j - 16) (P_0 + P_1 + P_2 + P_3+).
// The truncation error is ~2^-(8S+1) of the row maxima.
//
// A tcgen05.mma costs about the same whatever its N (measured: N = 32..128 and
// M = 64 or 128 all take ~88 cycles per instruction here), so the products are
// issued as few, wide instructions: the B slices are adjacent in shared memory,
// and A_t times B slices 0..3-t is one MMA of N = 64 (4 - t) whose column blocks
// are the accumulators of levels t..3. S = 4 takes 7 instructions per K step
// instead of 13, S = 5 takes 13 instead of 19.
//
// Data path: slices are stored pre-tiled in the canonical no-swizzle K-major
// UMMA layout (8-row x 16-byte core matrices, 64-row x 32-K tiles), so one
// cp.async.bulk per slice moves a chunk to shared memory. The GEMM kernel is
// persistent and warp-specialised: a producer warp streams K chunks of the
// CTA's output tiles through a ring of shared-memory stages, an MMA warp
// issues tcgen05.mma into one of two TMEM accumulator sets and commits to
// mbarriers, and sixteen epilogue warps drain the other set with tcgen05.ld
// and update C while the next group accumulates. Every wait is bounded: on
// timeout the kernel records an error, drains what it issued, releases TMEM
// and returns.
#include <math.h>
#include <stdint.h>

#include <algorithm>

#include "bulk.cuh"
#include "common.cuh"
#include "dfloat.cuh"
#include "model.cuh"

namespace gpgp {

constexpr int OZ_TK = 32;               // K chunk (one pipeline stage)
constexpr int OZ_GROUP = 8;             // chunks per exactly accumulated group (K = 256)
constexpr int OZ_TR = 64;               // rows per slice tile
constexpr int OZ_TILE = OZ_TR * OZ_TK;  // bf16 elements per slice tile (4 KB)
constexpr int OZ_BM = 128, OZ_BN = 64;  // output tile
constexpr int OZ_NACC = 4;              // accumulators: levels 0, 1, 2, >= 3
constexpr int OZ_EPI_WARPS = 16;  // four per TMEM lane quarter, 16 columns each
constexpr int OZ_EPI_COLS = OZ_BN / (OZ_EPI_WARPS / 4);
constexpr int OZ_THREADS = 32 * (2 + OZ_EPI_WARPS);  // producer, MMA, epilogue

// S slices per operand (8S-bit fixed point): levels t + u <= S are kept
// (S = 4: 13 products, truncation 2^-33; S = 5: 19 products, 2^-41).
template <int S>
struct OzCfg {
  static constexpr int A_SL = OZ_BM * OZ_TK * 2;  // bytes of one A slice chunk (8 KB)
  static constexpr int B_SL = OZ_BN * OZ_TK * 2;  // 4 KB
  static constexpr int STAGE = S * (A_SL + B_SL);
  static constexpr int NST = S == 4 ? 4 : 3;      // pipeline stages
  static constexpr int SMEM = NST * STAGE + 1024 + 1024;  // + barriers + alignment
  static constexpr uint32_t TMEM_COLS = 2 * OZ_NACC * OZ_BN;  // two accumulator sets
};

// ---------------------------------------------------------------------------
// split: FP64 rows -> S BF16 slices (canonical layout) + per-row exponents
// ---------------------------------------------------------------------------
// Element (r, k) of the logical rows x K operand is P[r + k*ld] (trans = 0)
// or P[k + r*ld] (trans = 1). Tiles: [slice][kc][rb], 64 rows x 32 K each
// (kc counts 32-wide chunks, 2 per 64-wide K block); within a tile, (r, k)
// lives at (r/8)*256 + (k/8)*64 + (r%8)*8 + (k%8) elements.
__device__ __forceinline__ double oz_elem(const double *P, int64_t ld, int trans, int64_t r,
                                          int64_t k, int64_t rows, int64_t K) {
  if (r >= rows || k >= K) return 0.0;
  return trans ? P[k + r * ld] : P[r + k * ld];
}

// Row exponents and slices are computed from the FP64 bit patterns with
// integer instructions only (the FP64 pipe of this part is slow).

// bf16 bits of q 2^-8t, |q| <= 256 (exact: at most 8 significant bits)
__device__ __forceinline__ uint32_t bf16_of_digit(int q, int t) {
  if (q == 0) return 0u;
  const uint32_t sgn = q < 0 ? 0x8000u : 0u;
  const uint32_t a = (uint32_t)(q < 0 ? -q : q);
  const int p = 31 - __clz(a);
  const uint32_t mant = p <= 7 ? ((a << (7 - p)) & 0x7Fu) : ((a >> (p - 7)) & 0x7Fu);
  return sgn | ((uint32_t)(127 + p - 8 * t) << 7) | mant;
}

// 8S-bit fixed point |x| 2^8S (rounded to nearest) of x = P 2^-e, as balanced
// base-256 digits d0..d(S-1) (|d0| <= 256, the others <= 128) carrying the sign of P
template <int S>
__device__ __forceinline__ void oz_digits(double v, int e, int d[S]) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(v);
  const int E = (int)((b >> 52) & 0x7FF);
  unsigned long long X = 0ull;
  if (E != 0 && E != 2047) {
    const unsigned long long mnt = (b & 0xFFFFFFFFFFFFFull) | (1ull << 52);
    const int rsh = 1075 + e - E - 8 * S;  // >= 13 because |v| < 2^e
    if (rsh < 64) X = (mnt + (1ull << (rsh - 1))) >> rsh;
  }
  int u[S];
#pragma unroll
  for (int t = 0; t < S; ++t) u[t] = (int)((X >> (8 * (S - 1 - t))) & 255ull);
  u[0] = (int)(X >> (8 * (S - 1)));
#pragma unroll
  for (int t = S - 1; t >= 1; --t)
    if (u[t] >= 128) {
      u[t] -= 256;
      u[t - 1] += 1;
    }
  const int sg = (b >> 63) ? -1 : 1;
#pragma unroll
  for (int t = 0; t < S; ++t) d[t] = sg * u[t];
}

// One-pass split: a block takes 32 rows, finds their maxima (coalesced for either
// layout: lanes over rows when columns are contiguous, over K when rows are),
// then writes every slice of those rows.
template <int S>
__global__ void __launch_bounds__(256) oz_split_kernel(const double *__restrict__ P, int64_t ld, int trans,
                                                       int64_t rows, int64_t K, int64_t nrb, int64_t nkb,
                                                       int *__restrict__ ex, uint16_t *__restrict__ sl,
                                                       int64_t sP, int64_t sE, int64_t sS) {
  P += blockIdx.y * sP;
  ex += blockIdx.y * sE;
  sl += blockIdx.y * sS;
  __shared__ unsigned long long part[8][32];
  __shared__ int exs[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t r0 = (int64_t)blockIdx.x * 32;
  if (!trans) {
    const int64_t r = r0 + lane;
    unsigned long long mx = 0ull;
    if (r < rows)
      for (int64_t k = warp; k < K; k += 8) {
        const unsigned long long b = (unsigned long long)__double_as_longlong(P[r + k * ld]) & 0x7FFFFFFFFFFFFFFFull;
        mx = b > mx ? b : mx;
      }
    part[warp][lane] = mx;
  } else {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int rl = warp * 4 + q;
      const int64_t r = r0 + rl;
      unsigned long long mx = 0ull;
      if (r < rows)
        for (int64_t k = lane; k < K; k += 32) {
          const unsigned long long b = (unsigned long long)__double_as_longlong(P[k + r * ld]) & 0x7FFFFFFFFFFFFFFFull;
          mx = b > mx ? b : mx;
        }
      for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long t = __shfl_xor_sync(0xffffffffu, mx, o);
        mx = t > mx ? t : mx;
      }
      if (lane == 0) part[0][rl] = mx;
    }
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    unsigned long long mx = part[0][lane];
    if (!trans)
#pragma unroll
      for (int w = 1; w < 8; ++w) mx = part[w][lane] > mx ? part[w][lane] : mx;
    // frexp exponent of the row maximum: max = 0.1m x 2^e; zero, subnormal or non-finite rows -> 0
    const int E = (int)(mx >> 52);
    const int e = (E == 0 || E == 2047) ? 0 : E - 1022;
    exs[lane] = e;
    if (r0 + lane < nrb * OZ_TR) ex[r0 + lane] = e;
  }
  __syncthreads();
  // The block's 32 rows go through shared memory 64 K at a time, read along the
  // operand's contiguous direction (rows for trans = 0, K for trans = 1), so that
  // the slices are written with consecutive lanes on consecutive rows in either
  // layout (four full 128-byte lines per store).
  __shared__ double T[32][65];
  const int64_t nkc = 2 * nkb;
  const int rl = threadIdx.x & 31, gl = threadIdx.x >> 5;  // row, 8-wide K group of the chunk
  const int64_t r = r0 + rl;
  const int e = exs[rl];
  for (int64_t kb0 = 0; kb0 < nkb * 64; kb0 += 64) {
    __syncthreads();
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int idx = threadIdx.x + 256 * q;
      const int ar = trans ? idx / 64 : idx % 32, ak = trans ? idx % 64 : idx / 32;
      T[ar][ak] = oz_elem(P, ld, trans, r0 + ar, kb0 + ak, rows, K);
    }
    __syncthreads();
    if (r >= nrb * OZ_TR) continue;
    const int64_t k0 = kb0 + 8 * gl;
    uint32_t packed[S][4];
#pragma unroll
    for (int j = 0; j < 8; j += 2) {
      int d0[S], d1[S];
      oz_digits<S>(T[rl][8 * gl + j], e, d0);
      oz_digits<S>(T[rl][8 * gl + j + 1], e, d1);
#pragma unroll
      for (int t = 0; t < S; ++t) packed[t][j / 2] = bf16_of_digit(d0[t], t) | (bf16_of_digit(d1[t], t) << 16);
    }
    const int64_t rb = r / OZ_TR, rr = r % OZ_TR;
    const int64_t kc = k0 / OZ_TK, kk = k0 % OZ_TK;
    const int64_t within = (rr / 8) * 256 + (kk / 8) * 64 + (rr % 8) * 8;
#pragma unroll
    for (int t = 0; t < S; ++t) {
      const int64_t tile = ((int64_t)t * nkc + kc) * nrb + rb;
      *reinterpret_cast<uint4 *>(sl + tile * OZ_TILE + within) =
          make_uint4(packed[t][0], packed[t][1], packed[t][2], packed[t][3]);
    }
  }
}

// Two-pass split for operands with too few 32-row groups to fill the GPU: pass 1
// takes the biased exponent field E of every element of 32 rows x 256 K and
// atomically maximises it per row (E is monotonic in |x|, so the row's largest E
// is that of its largest element; 0 and 2047 mark zero / subnormal and
// non-finite rows as in the one-pass kernel); pass 2 writes the slices of one
// 64-wide K block of 32 rows per CTA.
constexpr int OZ_EK = 256;  // K per pass-1 CTA

__global__ void __launch_bounds__(256) oz_rowexp_kernel(const double *__restrict__ P, int64_t ld, int trans,
                                                        int64_t rows, int64_t K, int *__restrict__ Emax,
                                                        int64_t sP, int64_t sM) {
  P += blockIdx.z * sP;
  Emax += blockIdx.z * sM;
  __shared__ int part[8][33];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t r0 = (int64_t)blockIdx.x * 32;
  const int64_t k0 = (int64_t)blockIdx.y * OZ_EK;
  const int64_t k1 = k0 + OZ_EK < K ? k0 + OZ_EK : K;
  if (!trans) {
    const int64_t r = r0 + lane;
    int mx = 0;
    if (r < rows)
      for (int64_t k = k0 + warp; k < k1; k += 8) {
        const int E = (int)(((unsigned long long)__double_as_longlong(P[r + k * ld]) >> 52) & 0x7FF);
        mx = E > mx ? E : mx;
      }
    part[warp][lane] = mx;
  } else {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int rl = warp * 4 + q;
      const int64_t r = r0 + rl;
      int mx = 0;
      if (r < rows)
        for (int64_t k = k0 + lane; k < k1; k += 32) {
          const int E = (int)(((unsigned long long)__double_as_longlong(P[k + r * ld]) >> 52) & 0x7FF);
          mx = E > mx ? E : mx;
        }
      for (int o = 16; o > 0; o >>= 1) {
        const int t = __shfl_xor_sync(0xffffffffu, mx, o);
        mx = t > mx ? t : mx;
      }
      if (lane == 0) part[0][rl] = mx;
    }
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    int mx = part[0][lane];
    if (!trans)
#pragma unroll
      for (int w = 1; w < 8; ++w) mx = part[w][lane] > mx ? part[w][lane] : mx;
    if (r0 + lane < rows && mx > 0) atomicMax(Emax + r0 + lane, mx);
  }
}

template <int S>
__global__ void __launch_bounds__(256) oz_slice_kernel(const double *__restrict__ P, int64_t ld, int trans,
                                                       int64_t rows, int64_t K, int64_t nrb, int64_t nkb,
                                                       const int *__restrict__ Emax, int *__restrict__ ex,
                                                       uint16_t *__restrict__ sl, int64_t sP, int64_t sE,
                                                       int64_t sS, int64_t sM) {
  P += blockIdx.z * sP;
  ex += blockIdx.z * sE;
  sl += blockIdx.z * sS;
  Emax += blockIdx.z * sM;
  __shared__ double T[32][65];
  const int64_t r0 = (int64_t)blockIdx.x * 32;
  const int rl = threadIdx.x & 31, gl = threadIdx.x >> 5;
  const int64_t r = r0 + rl;
  const int E = r < rows ? Emax[r] : 0;
  const int e = (E == 0 || E == 2047) ? 0 : E - 1022;
  if (blockIdx.y == 0 && gl == 0 && r < nrb * OZ_TR) ex[r] = e;
  const int64_t kb0 = (int64_t)blockIdx.y * 64;
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const int idx = threadIdx.x + 256 * q;
    const int ar = trans ? idx / 64 : idx % 32, ak = trans ? idx % 64 : idx / 32;
    T[ar][ak] = oz_elem(P, ld, trans, r0 + ar, kb0 + ak, rows, K);
  }
  __syncthreads();
  if (r >= nrb * OZ_TR) return;
  const int64_t k0 = kb0 + 8 * gl;
  uint32_t packed[S][4];
#pragma unroll
  for (int j = 0; j < 8; j += 2) {
    int d0[S], d1[S];
    oz_digits<S>(T[rl][8 * gl + j], e, d0);
    oz_digits<S>(T[rl][8 * gl + j + 1], e, d1);
#pragma unroll
    for (int t = 0; t < S; ++t) packed[t][j / 2] = bf16_of_digit(d0[t], t) | (bf16_of_digit(d1[t], t) << 16);
  }
  const int64_t nkc = 2 * nkb;
  const int64_t rb = r / OZ_TR, rr = r % OZ_TR;
  const int64_t kc = k0 / OZ_TK, kk = k0 % OZ_TK;
  const int64_t within = (rr / 8) * 256 + (kk / 8) * 64 + (rr % 8) * 8;
#pragma unroll
  for (int t = 0; t < S; ++t) {
    const int64_t tile = ((int64_t)t * nkc + kc) * nrb + rb;
    *reinterpret_cast<uint4 *>(sl + tile * OZ_TILE + within) =
        make_uint4(packed[t][0], packed[t][1], packed[t][2], packed[t][3]);
  }
}

// 64-row tiles of a split operand: one more than the rows need, rounded up to
// an even count, so that a 128-row A tile starting at any 64-row offset inside
// the operand stays inside the buffer.
int64_t oz_nrb(int64_t rows) {
  const int64_t t = (rows + OZ_TR - 1) / OZ_TR + 1;
  return (t + 1) / 2 * 2;
}

void oz_split_batched(cudaStream_t s, const double *P, int64_t ld, int64_t sP, int trans, int64_t rows,
                      int64_t K, OzSplit *out, int64_t batch) {
  const int64_t nrb = oz_nrb(rows);
  const int64_t nkb = (K + 63) / 64;
  out->rows = rows;
  out->K = K;
  out->nrb = nrb;
  out->nkb = nkb;
  const int64_t rows_pad = nrb * OZ_TR;
  const int64_t sE = out->bstride_ex, sS = out->bstride_sl;
  KTScope kts(GPGP_KPROF_OZ_SPLIT, s, 0.0);
  const int64_t groups = rows_pad / 32;
  if (groups * batch < 2 * (int64_t)device_sms() && nkb >= 2 && batch <= 65535) {
    // too few row groups for one CTA each to fill the GPU: two passes over a 2-D grid
    int *Emax = nullptr;
    GPGP_CUDA(cudaMallocAsync((void **)&Emax, (size_t)rows_pad * batch * sizeof(int), s));
    GPGP_CUDA(cudaMemsetAsync(Emax, 0, (size_t)rows_pad * batch * sizeof(int), s));
    dim3 g1((unsigned)groups, (unsigned)((K + OZ_EK - 1) / OZ_EK), (unsigned)batch);
    oz_rowexp_kernel<<<g1, 256, 0, s>>>(P, ld, trans, rows, K, Emax, sP, rows_pad);
    GPGP_CHECK_LAUNCH();
    dim3 g2((unsigned)groups, (unsigned)nkb, (unsigned)batch);
    if (out->S == 5)
      oz_slice_kernel<5><<<g2, 256, 0, s>>>(P, ld, trans, rows, K, nrb, nkb, Emax, out->ex, out->sl, sP, sE, sS,
                                            rows_pad);
    else
      oz_slice_kernel<4><<<g2, 256, 0, s>>>(P, ld, trans, rows, K, nrb, nkb, Emax, out->ex, out->sl, sP, sE, sS,
                                            rows_pad);
    GPGP_CHECK_LAUNCH();
    GPGP_CUDA(cudaFreeAsync(Emax, s));
    return;
  }
  dim3 g((unsigned)groups, (unsigned)batch);
  if (out->S == 5)
    oz_split_kernel<5><<<g, 256, 0, s>>>(P, ld, trans, rows, K, nrb, nkb, out->ex, out->sl, sP, sE, sS);
  else
    oz_split_kernel<4><<<g, 256, 0, s>>>(P, ld, trans, rows, K, nrb, nkb, out->ex, out->sl, sP, sE, sS);
  GPGP_CHECK_LAUNCH();
}

void oz_split(cudaStream_t s, const double *P, int64_t ld, int trans, int64_t rows, int64_t K,
              OzSplit *out) {
  oz_split_batched(s, P, ld, 0, trans, rows, K, out, 1);
}

size_t oz_split_bytes(int64_t rows, int64_t K, int S) {
  const int64_t nrb = oz_nrb(rows);
  const int64_t nkb = (K + 63) / 64;
  return (size_t)nrb * OZ_TR * sizeof(int) + 256 + (size_t)S * nkb * nrb * OZ_TR * 64 * 2;
}

void oz_split_bind(void *mem, int64_t rows, int64_t K, OzSplit *out, int S) {
  const int64_t nrb = oz_nrb(rows);
  (void)K;
  out->S = S;
  char *p = (char *)mem;
  out->ex = (int *)p;
  size_t exb = ((size_t)nrb * OZ_TR * sizeof(int) + 255) / 256 * 256;
  out->sl = (uint16_t *)(p + exb);
}

// ---------------------------------------------------------------------------
// PTX helpers (tcgen05, mbarrier, bulk copy)
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;  // descriptor version for tcgen05
  // base offset 0, lbo mode 0, layout type 0 (no swizzle)
  return d;
}

__device__ __forceinline__ void umma_bf16(uint32_t dtmem, uint64_t adesc, uint64_t bdesc,
                                          uint32_t idesc, uint32_t accum) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dtmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accum));
}

__device__ __forceinline__ void umma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
               : "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]),
        "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]),
        "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}

__device__ __forceinline__ void tmem_ld8(uint32_t taddr, uint32_t (&r)[8]) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                 "=r"(r[7])
               : "r"(taddr));
}

template <int NC>
__device__ __forceinline__ void tmem_ld(uint32_t taddr, uint32_t (&r)[NC]) {
  if constexpr (NC == 32) tmem_ld32(taddr, r);
  else tmem_ld16(taddr, r);
}

__device__ __forceinline__ void tmem_ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// double-float accumulation of v into (hi, lo) with an error-free TwoSum
__device__ __forceinline__ void df_add(float &hi, float &lo, float v) {
  const float s = __fadd_rn(hi, v);
  const float bp = __fsub_rn(s, hi);
  const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bp)), __fsub_rn(v, bp));
  hi = s;
  lo = __fadd_rn(lo, e);
}

// ---------------------------------------------------------------------------
// the GEMM: C = alpha * A B^T + beta * C over the given K range
// ---------------------------------------------------------------------------
struct OzGemmArgs {
  const uint16_t *a_sl;
  const int *a_ex;
  int64_t a_nrb, a_nkc, a_rb0;  // slice-tile geometry (32-wide K chunks); first 64-row tile
  const uint16_t *b_sl;
  const int *b_ex;
  int64_t b_nrb, b_nkc, b_rb0;
  int64_t M, N;
  int64_t kc0, kc1;  // 32-wide K chunks [kc0, kc1) of both operands
  int kmode;         // 0 all; 1 start at max(row,col); 2 start at col; 3 end after row
  double alpha, beta;
  double *C;
  int64_t ldc;
  int lower_only;
  int *err;
  const int *status;  // optional: skip a problem whose factorisation already failed
  int64_t a_bs_sl, a_bs_ex, b_bs_sl, b_bs_ex, c_bs;  // per-problem strides
  int64_t status_bs;
  int64_t gx, gy, batch;  // tile grid; tile L = (z gy + by) gx + bx
};

struct OzTile {
  int64_t z, row0, col0, c0, nch;
};

// The work of tile L (identical in every role): false when the tile is skipped
// (above the diagonal of a lower-only product, or its problem has failed)
__device__ __forceinline__ bool oz_tile_at(const OzGemmArgs &g, int64_t L, OzTile &t) {
  const int64_t per = g.gx * g.gy;
  t.z = L / per;
  const int64_t r = L - t.z * per;
  const int64_t by = r / g.gx, bx = r - by * g.gx;
  t.row0 = bx * OZ_BM;
  t.col0 = by * OZ_BN;
  if (g.lower_only && t.col0 > t.row0 + OZ_BM - 1) return false;
  if (g.status && *(volatile const int *)(g.status + t.z * g.status_bs) != 0) return false;
  const int64_t grow0 = g.a_rb0 * OZ_TR + t.row0, gcol0 = g.b_rb0 * OZ_TR + t.col0;
  int64_t k0 = g.kc0, k1 = g.kc1;
  if (g.kmode == 1) {
    const int64_t s0 = (grow0 > gcol0 ? grow0 : gcol0) / OZ_TK;
    k0 = k0 > s0 ? k0 : s0;
  }
  if (g.kmode == 2) {
    const int64_t s0 = gcol0 / OZ_TK;
    k0 = k0 > s0 ? k0 : s0;
  }
  if (g.kmode == 3) {
    const int64_t e0 = (grow0 + OZ_BM + OZ_TK - 1) / OZ_TK;
    k1 = k1 < e0 ? k1 : e0;
  }
  t.c0 = k0;
  t.nch = k1 > k0 ? k1 - k0 : 0;
  return true;
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

// Bounded wait that also gives up when another role has aborted.
__device__ __forceinline__ bool oz_wait(uint32_t bar, uint32_t parity, volatile int *abort_flag) {
  for (uint32_t it = 0; it < (1u << 24); ++it) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((it & 255u) == 255u && *abort_flag) return false;
  }
  return false;
}

template <int S>
// 576 threads: the register cap keeps the block inside one SM's register file
__global__ void __maxnreg__(96) oz_gemm_kernel(const OzGemmArgs g) {
  using Cfg = OzCfg<S>;
  constexpr int NST = Cfg::NST;
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t *bars = (uint64_t *)(smem + NST * Cfg::STAGE);
  __shared__ uint32_t tmem_base_sh;
  __shared__ int abort_sh;
  volatile int *abort_flag = &abort_sh;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // barriers: full[NST] (operands landed), empty[NST] (MMAs that read a stage done),
  // tfull[2] (an accumulator set is ready), tempty[2] (the epilogue drained it), drain
  const int FULL = 0, EMPTY = NST, TFULL = 2 * NST, TEMPTY = 2 * NST + 2, DRAIN = 2 * NST + 4;
  auto bar = [&](int i) { return smem_u32(&bars[i]); };
  if (threadIdx.x == 0) {
    for (int i = 0; i < NST; ++i) {
      mbar_init(bar(FULL + i), 1);
      mbar_init(bar(EMPTY + i), 1);
    }
    for (int i = 0; i < 2; ++i) {
      mbar_init(bar(TFULL + i), 1);
      mbar_init(bar(TEMPTY + i), OZ_EPI_WARPS);
    }
    mbar_init(bar(DRAIN), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    abort_sh = 0;
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tmem_base_sh)),
                 "r"(Cfg::TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_base_sh;
  const int64_t ntiles = g.gx * g.gy * g.batch;
  int last_full_parity[NST];
#pragma unroll
  for (int i = 0; i < NST; ++i) last_full_parity[i] = -1;
  bool mma_issued = false;

  if (warp == 0) {
    // ---- producer: K chunks of this CTA's tiles into the stage ring ----
    if (lane == 0) {
      int st = 0;
      uint32_t ph = 0;
      for (int64_t L = blockIdx.x; L < ntiles; L += gridDim.x) {
        OzTile t;
        if (!oz_tile_at(g, L, t) || t.nch == 0) continue;
        const uint16_t *a_sl = g.a_sl + t.z * g.a_bs_sl;
        const uint16_t *b_sl = g.b_sl + t.z * g.b_bs_sl;
        const int64_t arb = g.a_rb0 + t.row0 / OZ_TR, brb = g.b_rb0 + t.col0 / OZ_TR;
        for (int64_t c = 0; c < t.nch; ++c) {
          if (!oz_wait(bar(EMPTY + st), ph ^ 1u, abort_flag)) {
            if (!*abort_flag) atomicExch(g.err, 1);
            abort_sh = 1;
            goto producer_done;
          }
          const uint32_t base = smem_u32(smem + st * Cfg::STAGE);
          mbar_expect_tx(bar(FULL + st), Cfg::STAGE);
          const int64_t kc = t.c0 + c;
#pragma unroll
          for (int s = 0; s < S; ++s) {
            bulk_g2s(base + s * Cfg::A_SL, a_sl + (((int64_t)s * g.a_nkc + kc) * g.a_nrb + arb) * OZ_TILE,
                     Cfg::A_SL, bar(FULL + st));
            bulk_g2s(base + S * Cfg::A_SL + s * Cfg::B_SL,
                     b_sl + (((int64_t)s * g.b_nkc + kc) * g.b_nrb + brb) * OZ_TILE, Cfg::B_SL, bar(FULL + st));
          }
          last_full_parity[st] = (int)ph;
          if (++st == NST) {
            st = 0;
            ph ^= 1u;
          }
        }
      }
    producer_done:;
    }
  } else if (warp == 1) {
    // ---- MMA issuer ----
    if (lane == 0) {
      // D F32, A/B BF16, K-major both, M = 128; N is set per instruction
      const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(OZ_BM >> 4) << 24);
      // no-swizzle K-major: core matrices of 8 rows x 16 bytes; LBO steps K (128 B),
      // SBO steps 8 rows (8 x 32 K x 2 B = 512 B)
      const uint32_t lbo = 128u, sbo = 512u;
      int st = 0, b = 0;
      uint32_t ph = 0, tph[2] = {0u, 0u};
      for (int64_t L = blockIdx.x; L < ntiles; L += gridDim.x) {
        OzTile t;
        if (!oz_tile_at(g, L, t) || t.nch == 0) continue;
        uint32_t fresh = 0;  // 1 while the group's accumulators are still to be overwritten
        for (int64_t c = 0; c < t.nch; ++c) {
          const bool gstart = (c % OZ_GROUP) == 0;
          const bool gend = ((c + 1) % OZ_GROUP) == 0 || c == t.nch - 1;
          if (gstart) {
            if (!oz_wait(bar(TEMPTY + b), tph[b] ^ 1u, abort_flag)) {
              if (!*abort_flag) atomicExch(g.err, 2);
              abort_sh = 1;
              goto mma_done;
            }
            tc_fence_after();
            fresh = 1;
          }
          if (!oz_wait(bar(FULL + st), ph, abort_flag)) {
            if (!*abort_flag) atomicExch(g.err, 2);
            abort_sh = 1;
            goto mma_done;
          }
          tc_fence_after();
          const uint32_t abase = smem_u32(smem + st * Cfg::STAGE);
          const uint32_t bbase = abase + S * Cfg::A_SL;
          // Descriptors of the stage; slices and K steps are offsets in 16-byte units
          // (shared addresses stay below 2^18, so the 14-bit address field never carries).
          const uint64_t ad0 = umma_desc(abase, lbo, sbo), bd0 = umma_desc(bbase, lbo, sbo);
          const uint32_t d0 = tmem + (uint32_t)(b * OZ_NACC * OZ_BN);
#pragma unroll
          for (int kk = 0; kk < OZ_TK / 16; ++kk) {
#pragma unroll
            for (int ti = 0; ti < S; ++ti) {
              const uint64_t ad = ad0 + (uint64_t)((ti * Cfg::A_SL + kk * 256) >> 4);
              // The B slices lie back to back with one 8-row stride, so slices
              // 0..3-ti read as one operand of 64 (4 - ti) rows: a single MMA puts
              // A_ti B_u^T (level ti + u) into accumulators ti..3, which are adjacent
              // column blocks. Its first issue in a group overwrites all four.
              if (ti < OZ_NACC)
                umma_bf16(d0 + (uint32_t)(ti * OZ_BN), ad, bd0 + (uint64_t)((kk * 256) >> 4),
                          idesc | ((uint32_t)((OZ_NACC - ti) * OZ_BN >> 3) << 17),
                          (kk == 0 && ti == 0) ? (fresh ^ 1u) : 1u);
              // the remaining products of levels > 3 go one by one into the last accumulator
#pragma unroll
              for (int ui = ti < OZ_NACC ? OZ_NACC - ti : 0; ui < S; ++ui) {
                if (ti + ui > S) continue;
                umma_bf16(d0 + (uint32_t)((OZ_NACC - 1) * OZ_BN), ad,
                          bd0 + (uint64_t)((ui * Cfg::B_SL + kk * 256) >> 4),
                          idesc | ((uint32_t)(OZ_BN >> 3) << 17), 1u);
              }
            }
          }
          fresh = 0;
          mma_issued = true;
          umma_commit(bar(EMPTY + st));
          if (++st == NST) {
            st = 0;
            ph ^= 1u;
          }
          if (gend) {
            umma_commit(bar(TFULL + b));
            tph[b] ^= 1u;
            b ^= 1;
          }
        }
      }
    mma_done:;
    }
  } else {
    // ---- epilogue: warps 2..17 drain TMEM lanes 32 (warp % 4).., 16 columns each ----
    const int quarter = warp & 3, part = (warp - 2) >> 2;
    int b = 0;
    uint32_t tph[2] = {0u, 0u};
    // alpha and beta tests once, as integers (the FP64 pipe is the scarce unit)
    const bool unit = (g.alpha == 1.0 || g.alpha == -1.0) && (g.beta == 0.0 || g.beta == 1.0);
    const bool beta0 = g.beta == 0.0, beta1 = g.beta == 1.0;
    const uint32_t negmask = g.alpha < 0.0 ? 0x80000000u : 0u;
    for (int64_t L = blockIdx.x; L < ntiles; L += gridDim.x) {
      OzTile t;
      if (!oz_tile_at(g, L, t)) continue;
      const int64_t my_row = t.row0 + quarter * 32 + lane;
      const bool row_ok = my_row < g.M;
      const int64_t col_base = t.col0 + part * OZ_EPI_COLS;
      double *crow = g.C + t.z * g.c_bs + my_row;
      // this thread's C values, loaded before the accumulators are ready so that
      // the loads overlap the MMAs
      double cv[OZ_EPI_COLS];
#pragma unroll
      for (int j = 0; j < OZ_EPI_COLS; ++j)
        cv[j] = (row_ok && !beta0 && col_base + j < g.N) ? crow[(col_base + j) * g.ldc] : 0.0;
      if (t.nch == 0) {  // nothing accumulated: C = beta C
        if (row_ok && !beta1)
#pragma unroll
          for (int j = 0; j < OZ_EPI_COLS; ++j) {
            const int64_t col = col_base + j;
            if (col < g.N && !(g.lower_only && my_row < col)) crow[col * g.ldc] = g.beta * cv[j];
          }
        continue;
      }
      const int *a_ex = g.a_ex + t.z * g.a_bs_ex;
      const int *b_ex = g.b_ex + t.z * g.b_bs_ex + g.b_rb0 * OZ_TR;
      const int ea = row_ok ? a_ex[g.a_rb0 * OZ_TR + my_row] : 0;
      const int64_t ngr = (t.nch + OZ_GROUP - 1) / OZ_GROUP;
      // the tile's sum over its K groups, in double-float (level-0 units)
      float hi[OZ_EPI_COLS], lo[OZ_EPI_COLS];
#pragma unroll
      for (int j = 0; j < OZ_EPI_COLS; ++j) hi[j] = lo[j] = 0.f;
      for (int64_t gi = 0; gi < ngr; ++gi) {
        int ok = 1;
        if (lane == 0) ok = oz_wait(bar(TFULL + b), tph[b], abort_flag) ? 1 : 0;
        ok = __shfl_sync(0xffffffffu, ok, 0);
        if (!ok) {
          if (lane == 0) {
            if (!*abort_flag) atomicExch(g.err, 3);
            abort_sh = 1;
          }
          goto epi_done;
        }
        tc_fence_after();
#pragma unroll
        for (int cb = 0; cb < OZ_EPI_COLS / 8; ++cb) {
          uint32_t r[OZ_NACC][8];
#pragma unroll
          for (int acc = 0; acc < OZ_NACC; ++acc)
            tmem_ld8(tmem + ((uint32_t)(quarter * 32) << 16) +
                         (uint32_t)((b * OZ_NACC + acc) * OZ_BN + part * OZ_EPI_COLS + cb * 8),
                     r[acc]);
          tmem_ld_wait();
#pragma unroll
          for (int j = 0; j < 8; ++j) {
#pragma unroll
            for (int acc = 0; acc < OZ_NACC; ++acc) df_add(hi[cb * 8 + j], lo[cb * 8 + j], __uint_as_float(r[acc][j]));
          }
        }
        // every load of this set has completed: hand it back to the MMA warp
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(bar(TEMPTY + b));
        tph[b] ^= 1u;
        b ^= 1;
      }
      // C = alpha 2^(e_i + f_j - 16) (hi + lo) + beta C
      if (row_ok) {
#pragma unroll
        for (int j = 0; j < OZ_EPI_COLS; ++j) {
          const int64_t col = col_base + j;
          if (col < g.N && !(g.lower_only && my_row < col)) {
            const int sh = ea + b_ex[col] - 16;
            double out;
            if (unit) {
              // the sign of alpha goes onto the FP32 pair
              const float h = __uint_as_float(__float_as_uint(hi[j]) ^ negmask);
              const float l = __uint_as_float(__float_as_uint(lo[j]) ^ negmask);
              const double v = df2d_scaled(h, l, sh);
              out = beta0 ? v : cv[j] + v;
            } else {
              const double v = f2d_scaled(hi[j], sh) + f2d_scaled(lo[j], sh);
              out = beta0 ? g.alpha * v : fma(g.alpha, v, g.beta * cv[j]);
            }
            crow[col * g.ldc] = out;
          }
        }
      }
    }
  epi_done:;
  }

  __syncthreads();
  if (abort_sh) {
    // a wait ran out: let what was issued land (bounded) before the shared memory
    // and TMEM are released
    if (warp == 1 && lane == 0 && mma_issued) {
      umma_commit(bar(DRAIN));
      mbar_wait_bounded(bar(DRAIN), 0);
    }
    if (warp == 0 && lane == 0)
      for (int i = 0; i < NST; ++i)
        if (last_full_parity[i] >= 0) mbar_wait_bounded(bar(FULL + i), (uint32_t)last_full_parity[i]);
  }
  __syncthreads();
  if (warp == 1) {
    __syncwarp();
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(Cfg::TMEM_COLS));
  }
}

thread_local int tl_oz_grid_cap = 0;

static int oz_sm_count() { return device_sms(); }

void oz_gemm_batched(cudaStream_t s, const OzSplit &A, int64_t a_row0, const OzSplit &B, int64_t b_row0,
                     int64_t M, int64_t N, int64_t kc0, int64_t kc1, int kmode, double alpha,
                     double beta, double *C, int64_t ldc, int64_t sC, bool lower_only, int *err,
                     const int *status, int64_t status_bs, int64_t batch) {
  if (M <= 0 || N <= 0 || batch <= 0) return;
  if (A.S != B.S) throw CudaError{cudaErrorInvalidValue, "oz_gemm: operands split to different slice counts", __LINE__};
  static PerDevice attr;
  per_device(attr, [] {
    GPGP_CUDA(cudaFuncSetAttribute(oz_gemm_kernel<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, OzCfg<4>::SMEM));
    GPGP_CUDA(cudaFuncSetAttribute(oz_gemm_kernel<5>, cudaFuncAttributeMaxDynamicSharedMemorySize, OzCfg<5>::SMEM));
    return 1;
  });
  OzGemmArgs g;
  g.a_sl = A.sl;
  g.a_ex = A.ex;
  g.a_nrb = A.nrb;
  g.a_nkc = 2 * A.nkb;
  g.a_rb0 = a_row0 / OZ_TR;
  g.b_sl = B.sl;
  g.b_ex = B.ex;
  g.b_nrb = B.nrb;
  g.b_nkc = 2 * B.nkb;
  g.b_rb0 = b_row0 / OZ_TR;
  g.M = M;
  g.N = N;
  // callers count K in 64-wide blocks; the kernel in 32-wide chunks
  g.kc0 = 2 * kc0;
  g.kc1 = std::min<int64_t>(2 * kc1, std::min(g.a_nkc, g.b_nkc));
  g.kmode = kmode;
  g.alpha = alpha;
  g.beta = beta;
  g.C = C;
  g.ldc = ldc;
  g.lower_only = lower_only ? 1 : 0;
  g.err = err;
  g.status = status;
  g.a_bs_sl = A.bstride_sl;
  g.a_bs_ex = A.bstride_ex;
  g.b_bs_sl = B.bstride_sl;
  g.b_bs_ex = B.bstride_ex;
  g.c_bs = sC;
  g.status_bs = status_bs;
  g.gx = (M + OZ_BM - 1) / OZ_BM;
  g.gy = (N + OZ_BN - 1) / OZ_BN;
  g.batch = batch;
  const int64_t ntiles = g.gx * g.gy * batch;
  const int64_t cap = tl_oz_grid_cap > 0 ? std::min(tl_oz_grid_cap, oz_sm_count()) : oz_sm_count();
  const int64_t grid = std::min<int64_t>(ntiles, cap);
  double fl = 0.0;
  if (tl_kt) {
    // executed MMA arithmetic of the tiles the launch runs (the kernel's own tile
    // skipping and K ranges; failed problems are not known on the host)
    const int prods = A.S == 5 ? 19 : 13;
    for (int64_t bx = 0; bx < g.gx; ++bx)
      for (int64_t by = 0; by < g.gy; ++by) {
        const int64_t row0 = bx * OZ_BM, col0 = by * OZ_BN;
        if (lower_only && col0 > row0 + OZ_BM - 1) continue;
        const int64_t grow0 = g.a_rb0 * OZ_TR + row0, gcol0 = g.b_rb0 * OZ_TR + col0;
        int64_t k0 = g.kc0, k1 = g.kc1;
        if (kmode == 1) k0 = std::max(k0, std::max(grow0, gcol0) / OZ_TK);
        if (kmode == 2) k0 = std::max(k0, gcol0 / OZ_TK);
        if (kmode == 3) k1 = std::min(k1, (grow0 + OZ_BM + OZ_TK - 1) / OZ_TK);
        if (k1 > k0) fl += 2.0 * OZ_BM * OZ_BN * OZ_TK * (double)(k1 - k0) * prods;
      }
    fl *= (double)batch;
  }
  {
    KTScope kts(GPGP_KPROF_OZ_GEMM, s, fl);
    if (A.S == 5)
      oz_gemm_kernel<5><<<(unsigned)grid, OZ_THREADS, OzCfg<5>::SMEM, s>>>(g);
    else
      oz_gemm_kernel<4><<<(unsigned)grid, OZ_THREADS, OzCfg<4>::SMEM, s>>>(g);
  }
  GPGP_CHECK_LAUNCH();
}

int oz_sms() { return oz_sm_count(); }

void oz_gemm(cudaStream_t s, const OzSplit &A, int64_t a_row0, const OzSplit &B, int64_t b_row0,
             int64_t M, int64_t N, int64_t kc0, int64_t kc1, int kmode, double alpha, double beta,
             double *C, int64_t ldc, bool lower_only, int *err, const int *status) {
  oz_gemm_batched(s, A, a_row0, B, b_row0, M, N, kc0, kc1, kmode, alpha, beta, C, ldc, 0, lower_only,
                  err, status, 0, 1);
}


}  // namespace gpgp

// ---------------------------------------------------------------------------
// bounded-wait self-test: an mbarrier that is never completed (two arrivals
// expected, one made), polled with the same loop as the GEMM's waits but with a
// caller-chosen bound; the kernel records the timeout and returns
// ---------------------------------------------------------------------------
namespace gpgp {
__global__ void wait_selftest_kernel(uint32_t polls, int *err) {
  __shared__ uint64_t bar;
  __shared__ int abort_sh;
  if (threadIdx.x == 0) {
    mbar_init(smem_u32(&bar), 2);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    abort_sh = 0;
    mbar_arrive(smem_u32(&bar));
    bool done = false;
    for (uint32_t it = 0; it < polls && !done; ++it) done = mbar_try_wait(smem_u32(&bar), 0);
    if (!done) atomicExch(err, 4);
  }
  __syncthreads();
}
}  // namespace gpgp

extern "C" gpgp_status gpgp_wait_selftest(gpgp_ctx *ctx, int32_t polls) {
  if (!ctx || polls < 1) return GPGP_EINVAL;
  return gpgp::guarded(ctx, [&]() -> gpgp_status {
    GPGP_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    gpgp::IBuf err;
    err.alloc(s, 1);
    GPGP_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), s));
    gpgp::wait_selftest_kernel<<<1, 32, 0, s>>>((uint32_t)polls, err.p);
    GPGP_CHECK_LAUNCH();
    int h = 0;
    GPGP_CUDA(cudaMemcpyAsync(&h, err.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    GPGP_CUDA(cudaStreamSynchronize(s));
    if (h) return gpgp::fail(ctx, GPGP_ETIMEOUT, "a bounded device wait ran out (self-test)");
    return GPGP_OK;
  });
}
