// Mixed-precision dense kernels: FP64-accurate products on the tcgen05
// tensor cores through exact BF16 slicing (an Ozaki-style split).
//
// Every operand row is scaled by a power of two so that its largest entry is
// in [0.5, 1) and then cut into four 8-bit fixed-point slices
//   x = 2^e * sum_t q_t 2^-8(t+1),  q_t integers in [-256, 256]
// which BF16 holds exactly. A product of two slices is an integer below 2^16,
// so the level-0 and level-1 dot products of up to 256 terms stay below 2^24
// and the FP32 accumulators of tcgen05.mma hold them exactly. The 13 slice
// pairs with t + u <= 4 go into five level accumulators in TMEM; after every
// 256-wide K group the levels are added into double-float (hi, lo) FP32
// registers, and the result is written once in FP64:
//   (A B^T)_ij = 2^(e_i + f_j - 16) sum_l 2^-8l P_l.
// The truncation error is ~2^-33 of the row maxima, far below what the FP64
// log-determinant and iterative refinement need for 1e-8 evidence accuracy.
//
// Data path: slices are stored pre-tiled in the canonical no-swizzle K-major
// UMMA layout (8-row x 16-byte core matrices), so one cp.async.bulk per slice
// tile moves them to shared memory; one elected thread issues the MMAs and a
// tcgen05.commit arrives on an mbarrier; all eight warps drain TMEM with
// tcgen05.ld. Every wait is bounded: on timeout the kernel records an error,
// releases TMEM and returns.
#include <math.h>
#include <stdint.h>

#include <algorithm>

#include "common.cuh"

namespace gpgp {

constexpr int OZ_TK = 64;           // K chunk
// Chunks accumulated in TMEM before a flush: level-0 and level-1 sums stay below
// 2^24 (exact in FP32) for 4 x 64 = 256 products; deeper levels may round, but
// their rounding is below 2^-40 of the result.
constexpr int OZ_GROUP = 4;
constexpr int OZ_TR = 64;           // rows per slice tile
constexpr int OZ_TILE = OZ_TR * OZ_TK;  // bf16 elements per slice tile (8 KB)
constexpr int OZ_BM = 128;

// S slices per operand (8S-bit fixed point): levels t + u <= S are kept
// (S = 4: 13 products, truncation 2^-33; S = 5: 19 products, 2^-41). The
// tile is 128 x 64 for S = 4 and 128 x 32 for S = 5 so that two pipeline
// stages of operands fit in shared memory.
template <int S>
struct OzCfg {
  static constexpr int LEVELS = S + 1;
  static constexpr int BN = S == 4 ? 64 : 32;
  static constexpr int A_STAGE = S * 2 * OZ_TILE * 2;  // S slices x 128 rows x 64 K x 2 B
  static constexpr int B_TILE = BN * OZ_TK * 2;        // one slice of BN rows
  static constexpr int B_STAGE = S * B_TILE;
  static constexpr int STAGE = A_STAGE + B_STAGE;
  static constexpr int SMEM = 2 * STAGE + 1024;
  static constexpr uint32_t TMEM_COLS = LEVELS * BN <= 256 ? 256u : 512u;
  static constexpr int CPT = BN / 2;  // accumulator columns per epilogue thread
};


// ---------------------------------------------------------------------------
// split: FP64 rows -> 4 BF16 slices (canonical layout) + per-row exponents
// ---------------------------------------------------------------------------
// Element (r, k) of the logical rows x K operand is P[r + k*ld] (trans = 0)
// or P[k + r*ld] (trans = 1). Tiles: [slice][kb][rb], 64 x 64 each; within a
// tile, (r, k) lives at (r/8)*512 + (k/8)*64 + (r%8)*8 + (k%8) elements.
__device__ __forceinline__ double oz_elem(const double *P, int64_t ld, int trans, int64_t r,
                                          int64_t k, int64_t rows, int64_t K) {
  if (r >= rows || k >= K) return 0.0;
  return trans ? P[k + r * ld] : P[r + k * ld];
}

// Row exponents and slices are computed from the FP64 bit patterns with
// integer instructions only (the FP64 pipe of this part is slow).

__global__ void oz_rowexp_kernel(const double *__restrict__ P, int64_t ld, int trans, int64_t rows,
                                 int64_t K, int64_t rows_pad, int *__restrict__ ex, int64_t sP,
                                 int64_t sE) {
  P += blockIdx.y * sP;  // batched: problem blockIdx.y
  ex += blockIdx.y * sE;
  // one warp per row: the largest |P| by an unsigned compare of the sign-cleared bits
  const int lane = threadIdx.x & 31;
  const int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (r >= rows_pad) return;
  unsigned long long mx = 0ull;
  if (r < rows)
    for (int64_t k = lane; k < K; k += 32) {
      const unsigned long long b =
          (unsigned long long)__double_as_longlong(trans ? P[k + r * ld] : P[r + k * ld]) & 0x7FFFFFFFFFFFFFFFull;
      mx = b > mx ? b : mx;
    }
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long t = __shfl_xor_sync(0xffffffffu, mx, o);
    mx = t > mx ? t : mx;
  }
  if (lane == 0) {
    // frexp exponent of the row maximum: max = 0.1m x 2^e; zero, subnormal or non-finite rows -> 0
    const int E = (int)(mx >> 52);
    ex[r] = (E == 0 || E == 2047) ? 0 : E - 1022;
  }
}

// bf16 bits of the integer s * q, |q| <= 256
__device__ __forceinline__ uint32_t bf16_of_digit(int q) {
  if (q == 0) return 0u;
  const uint32_t sgn = q < 0 ? 0x8000u : 0u;
  const uint32_t a = (uint32_t)(q < 0 ? -q : q);
  const int p = 31 - __clz(a);
  const uint32_t mant = p <= 7 ? ((a << (7 - p)) & 0x7Fu) : ((a >> (p - 7)) & 0x7Fu);
  return sgn | ((uint32_t)(127 + p) << 7) | mant;
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

template <int S>
__global__ void oz_slice_kernel(const double *__restrict__ P, int64_t ld, int trans, int64_t rows,
                                int64_t K, int64_t nrb, int64_t nkb, const int *__restrict__ ex,
                                uint16_t *__restrict__ sl, int64_t sP, int64_t sE, int64_t sS) {
  P += blockIdx.y * sP;  // batched: problem blockIdx.y
  ex += blockIdx.y * sE;
  sl += blockIdx.y * sS;
  // thread per (row, 8-wide K group): writes 16 bytes per slice
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t rows_pad = nrb * OZ_TR;
  const int64_t ngroups = nkb * (OZ_TK / 8);
  if (tid >= rows_pad * ngroups) return;
  const int64_t r = trans ? tid / ngroups : tid % rows_pad;
  const int64_t g = trans ? tid % ngroups : tid / rows_pad;
  const int64_t k0 = g * 8;
  const int e = ex[r];
  uint32_t packed[S][4];
#pragma unroll
  for (int j = 0; j < 8; j += 2) {
    int d0[S], d1[S];
    oz_digits<S>(oz_elem(P, ld, trans, r, k0 + j, rows, K), e, d0);
    oz_digits<S>(oz_elem(P, ld, trans, r, k0 + j + 1, rows, K), e, d1);
#pragma unroll
    for (int t = 0; t < S; ++t) packed[t][j / 2] = bf16_of_digit(d0[t]) | (bf16_of_digit(d1[t]) << 16);
  }
  const int64_t rb = r / OZ_TR, rr = r % OZ_TR;
  const int64_t kb = k0 / OZ_TK, kk = k0 % OZ_TK;
  const int64_t within = (rr / 8) * 512 + (kk / 8) * 64 + (rr % 8) * 8;
#pragma unroll
  for (int t = 0; t < S; ++t) {
    const int64_t tile = ((int64_t)t * nkb + kb) * nrb + rb;
    uint4 v = make_uint4(packed[t][0], packed[t][1], packed[t][2], packed[t][3]);
    *reinterpret_cast<uint4 *>(sl + tile * OZ_TILE + within) = v;
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
  const int64_t nkb = (K + OZ_TK - 1) / OZ_TK;
  out->rows = rows;
  out->K = K;
  out->nrb = nrb;
  out->nkb = nkb;
  const int64_t rows_pad = nrb * OZ_TR;
  const int64_t sE = out->bstride_ex, sS = out->bstride_sl;
  {
    const int64_t threads = rows_pad * 32;
    dim3 g((unsigned)((threads + 255) / 256), (unsigned)batch);
    oz_rowexp_kernel<<<g, 256, 0, s>>>(P, ld, trans, rows, K, rows_pad, out->ex, sP, sE);
    GPGP_CHECK_LAUNCH();
  }
  {
    const int64_t threads = rows_pad * nkb * (OZ_TK / 8);
    dim3 g((unsigned)((threads + 255) / 256), (unsigned)batch);
    if (out->S == 5)
      oz_slice_kernel<5><<<g, 256, 0, s>>>(P, ld, trans, rows, K, nrb, nkb, out->ex, out->sl, sP, sE, sS);
    else
      oz_slice_kernel<4><<<g, 256, 0, s>>>(P, ld, trans, rows, K, nrb, nkb, out->ex, out->sl, sP, sE, sS);
    GPGP_CHECK_LAUNCH();
  }
}

void oz_split(cudaStream_t s, const double *P, int64_t ld, int trans, int64_t rows, int64_t K,
              OzSplit *out) {
  oz_split_batched(s, P, ld, 0, trans, rows, K, out, 1);
}

size_t oz_split_bytes(int64_t rows, int64_t K, int S) {
  const int64_t nrb = oz_nrb(rows);
  const int64_t nkb = (K + OZ_TK - 1) / OZ_TK;
  return (size_t)nrb * OZ_TR * sizeof(int) + 256 + (size_t)S * nkb * nrb * OZ_TILE * 2;
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
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait: returns false after ~2^24 polls (about a second or more).
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity) {
  for (uint32_t it = 0; it < (1u << 24); ++it)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void *src, uint32_t bytes,
                                         uint32_t bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
      "l"(src), "r"(bytes), "r"(bar)
      : "memory");
}

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

template <int NC>
__device__ __forceinline__ void tmem_ld(uint32_t taddr, uint32_t (&r)[NC]) {
  if constexpr (NC == 32) tmem_ld32(taddr, r);
  else tmem_ld16(taddr, r);
}

__device__ __forceinline__ void tmem_ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// (double)f * 2^sh, exact, by moving the float's fields into a double: the
// float exponent is rebiased and sh added; zero and out-of-range cases take ldexp
__device__ __forceinline__ double f2d_scaled(float f, int sh) {
  const uint32_t b = __float_as_uint(f);
  const uint32_t ef = (b >> 23) & 0xFFu;
  if (ef == 0u || ef == 0xFFu) return ldexp((double)f, sh);
  const int ed = (int)ef - 127 + 1023 + sh;
  if (ed <= 0 || ed >= 2047) return ldexp((double)f, sh);
  const unsigned long long db = ((unsigned long long)(b >> 31) << 63) |
                                ((unsigned long long)ed << 52) |
                                ((unsigned long long)(b & 0x7FFFFFu) << 29);
  return __longlong_as_double((long long)db);
}

// double-float accumulation of v into (hi, lo) with an error-free TwoSum
__device__ __forceinline__ void df_add(float &hi, float &lo, float v) {
  const float s = __fadd_rn(hi, v);
  const float bp = __fsub_rn(s, hi);
  const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bp)), __fsub_rn(v, bp));
  hi = s;
  lo = __fadd_rn(lo, e);
}

// ---------------------------------------------------------------------------
// the GEMM: C = alpha * A B^T + beta * C over the given K-chunk range
// ---------------------------------------------------------------------------
struct OzGemmArgs {
  const uint16_t *a_sl;
  const int *a_ex;
  int64_t a_nrb, a_nkb, a_rb0;  // slice-tile geometry; first 64-row tile of this operand
  const uint16_t *b_sl;
  const int *b_ex;
  int64_t b_nrb, b_nkb, b_rb0;
  int64_t M, N;
  int64_t kc0, kc1;  // K chunks [kc0, kc1) of both operands
  int kmode;         // 0 all; 1 start at max(row,col)/64; 2 start at col/64; 3 end at row/64 + 2
  double alpha, beta;
  double *C;
  int64_t ldc;
  int lower_only;
  int *err;
  const int *status;  // optional: skip all work when a factorisation already failed
  int64_t a_bs_sl, a_bs_ex, b_bs_sl, b_bs_ex, c_bs;  // batch strides (problem blockIdx.z)
  int64_t status_bs;
};

template <int S>
__global__ void __launch_bounds__(256, 1) oz_gemm_kernel(const OzGemmArgs g) {
  using Cfg = OzCfg<S>;
  constexpr int BN = Cfg::BN, CPT = Cfg::CPT;
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  // align the dynamic shared memory base to 1024 bytes
  uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  const int tid = threadIdx.x;
  const int warp = tid >> 5, lane = tid & 31;
  const int64_t row0 = (int64_t)blockIdx.x * OZ_BM;
  const int64_t col0 = (int64_t)blockIdx.y * BN;
  if (g.lower_only && col0 > row0 + OZ_BM - 1) return;
  const int64_t zb = blockIdx.z;
  const uint16_t *a_sl = g.a_sl + zb * g.a_bs_sl;
  const int *a_ex = g.a_ex + zb * g.a_bs_ex;
  const uint16_t *b_sl = g.b_sl + zb * g.b_bs_sl;
  const int *b_ex = g.b_ex + zb * g.b_bs_ex;
  double *Cz = g.C + zb * g.c_bs;

  // K-chunk range of this tile
  const int64_t grow0 = g.a_rb0 * OZ_TR + row0;  // absolute operand row of the tile
  const int64_t gcol0 = g.b_rb0 * OZ_TR + col0;
  int64_t kc0 = g.kc0, kc1 = g.kc1;
  if (g.kmode == 1) {
    const int64_t s0 = (grow0 > gcol0 ? grow0 : gcol0) / OZ_TK;
    kc0 = kc0 > s0 ? kc0 : s0;
  }
  if (g.kmode == 2) {
    const int64_t s0 = gcol0 / OZ_TK;
    kc0 = kc0 > s0 ? kc0 : s0;
  }
  if (g.kmode == 3) {
    const int64_t e0 = (grow0 + OZ_BM + OZ_TK - 1) / OZ_TK;
    kc1 = kc1 < e0 ? kc1 : e0;
  }
  if (g.status && *(volatile const int *)(g.status + blockIdx.z * g.status_bs) != 0) return;
  const int64_t nch = kc1 > kc0 ? kc1 - kc0 : 0;

  uint64_t *bars = (uint64_t *)(smem + 2 * Cfg::STAGE);
  __shared__ uint32_t tmem_base_sh;
  __shared__ int abort_sh;
  // full[s]: operands of the chunk in stage s landed; empty[s]: the MMAs that read
  // stage s completed; flush: the MMAs of a flush group completed
  const uint32_t full0 = smem_u32(&bars[0]), full1 = smem_u32(&bars[1]);
  const uint32_t empty0 = smem_u32(&bars[2]), empty1 = smem_u32(&bars[3]);
  const uint32_t flushb = smem_u32(&bars[4]);
  if (tid == 0) {
    mbar_init(full0, 1);
    mbar_init(full1, 1);
    mbar_init(empty0, 1);
    mbar_init(empty1, 1);
    mbar_init(flushb, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    abort_sh = 0;
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tmem_base_sh)),
                 "r"(Cfg::TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_base_sh;

  // operand tile addresses for chunk c (global)
  auto a_tile = [&](int s, int64_t kc) {
    return a_sl + (((int64_t)s * g.a_nkb + kc) * g.a_nrb + g.a_rb0 + 2 * blockIdx.x) * OZ_TILE;
  };
  // a BN-row part of a 64-row slice tile is contiguous (rows are the outer index)
  auto b_tile = [&](int s, int64_t kc) {
    return b_sl + (((int64_t)s * g.b_nkb + kc) * g.b_nrb + g.b_rb0 + col0 / OZ_TR) * OZ_TILE +
           (col0 % OZ_TR) * OZ_TK;
  };
  auto load_stage = [&](int st, int64_t kc) {
    const uint32_t base = smem_u32(smem + st * Cfg::STAGE);
    const uint32_t bar = st ? full1 : full0;
    mbar_expect_tx(bar, Cfg::STAGE);
    for (int s = 0; s < S; ++s) {
      bulk_g2s(base + s * (2 * OZ_TILE * 2), a_tile(s, kc), 2 * OZ_TILE * 2, bar);
      bulk_g2s(base + Cfg::A_STAGE + s * Cfg::B_TILE, b_tile(s, kc), Cfg::B_TILE, bar);
    }
  };

  if (tid == 0 && nch > 0) load_stage(0, kc0);

  // instruction descriptor: D F32, A/B BF16, K-major both, N = BN, M = 128
  const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) |
                         ((uint32_t)(OZ_BM >> 4) << 24);
  // no-swizzle K-major operands: 8 x 16-byte core matrices, the leading byte
  // offset steps K (128 B), the stride byte offset steps 8 rows (1024 B)
  const uint32_t lbo = 128u, sbo = 1024u;

  // epilogue ownership: warp w reads TMEM lanes 32*(w%4).., columns CPT*(w/4)..
  const int quarter = warp & 3, half = warp >> 2;
  const int64_t my_row = row0 + quarter * 32 + lane;
  float hi[CPT], lo[CPT];
#pragma unroll
  for (int c = 0; c < CPT; ++c) hi[c] = lo[c] = 0.f;

  bool ok = true;
  int nflush = 0;
  for (int64_t c = 0; c < nch; ++c) {
    const int st = (int)(c & 1);
    const bool group_start = (c % OZ_GROUP) == 0;
    const bool flush = ((c + 1) % OZ_GROUP) == 0 || c == nch - 1;
    if (tid == 0) {
      bool good = mbar_wait_bounded(st ? full1 : full0, (uint32_t)((c >> 1) & 1));
      if (good) {
        tc_fence_after();
        const uint32_t abase = smem_u32(smem + st * Cfg::STAGE);
        const uint32_t bbase = abase + Cfg::A_STAGE;
        int first[Cfg::LEVELS];
#pragma unroll
        for (int l = 0; l < Cfg::LEVELS; ++l) first[l] = group_start ? 1 : 0;
#pragma unroll
        for (int t = 0; t < S; ++t) {
#pragma unroll
          for (int u = 0; u < S; ++u) {
            const int lev = t + u;
            if (lev >= Cfg::LEVELS) continue;
#pragma unroll
            for (int kk = 0; kk < OZ_TK / 16; ++kk) {
              const uint64_t ad = umma_desc(abase + t * (2 * OZ_TILE * 2) + kk * 2 * 128, lbo, sbo);
              const uint64_t bd = umma_desc(bbase + u * Cfg::B_TILE + kk * 2 * 128, lbo, sbo);
              umma_bf16(tmem + lev * BN, ad, bd, idesc, first[lev] ? 0u : 1u);
              first[lev] = 0;
            }
          }
        }
        umma_commit(st ? empty1 : empty0);
        if (flush) umma_commit(flushb);
        // refill the other stage with chunk c + 1 once the MMAs of chunk c - 1 are done
        if (c + 1 < nch) {
          if (c >= 1) good = mbar_wait_bounded(st ? empty0 : empty1, (uint32_t)(((c - 1) >> 1) & 1));
          if (good) load_stage(st ^ 1, kc0 + c + 1);
        }
      }
      if (!good) {
        atomicExch(g.err, 1);
        abort_sh = 1;
      }
    }
    if (flush) {
      __syncthreads();
      if (abort_sh) {
        ok = false;
        break;
      }
      const bool waited = mbar_wait_bounded(flushb, (uint32_t)(nflush & 1));
      if (__syncthreads_or(!waited)) {
        if (tid == 0) atomicExch(g.err, 2);
        ok = false;
        break;
      }
      ++nflush;
      tc_fence_after();
#pragma unroll 1
      for (int lev = 0; lev < Cfg::LEVELS; ++lev) {
        uint32_t r[CPT];
        tmem_ld<CPT>(tmem + ((uint32_t)(quarter * 32) << 16) + lev * BN + half * CPT, r);
        tmem_ld_wait();
        const float sc = __uint_as_float((uint32_t)(127 - 8 * lev) << 23);  // 2^-8lev
#pragma unroll
        for (int j = 0; j < CPT; ++j) df_add(hi[j], lo[j], __uint_as_float(r[j]) * sc);
      }
      tc_fence_before();
      __syncthreads();
    } else if (c % 8 == 7) {
      // keep abort visible between flushes without a barrier per chunk
      __syncthreads();
      if (abort_sh) {
        ok = false;
        break;
      }
    }
  }
  __syncthreads();
  if (!ok && tid == 0) {
    // a wait ran out: give in-flight MMAs and bulk copies a bounded chance to land
    // before the shared memory and TMEM are released
    mbar_wait_bounded(flushb, (uint32_t)(nflush & 1));
    mbar_wait_bounded(empty0, 0);
    mbar_wait_bounded(empty1, 0);
    mbar_wait_bounded(full0, 0);
    mbar_wait_bounded(full1, 0);
  }
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(Cfg::TMEM_COLS));
  }
  if (!ok) return;
  // FP64 epilogue: C = alpha * 2^(e_i + f_j - 16) (hi + lo) + beta * C, with the
  // float -> double conversion and the power of two done on the bit patterns
  if (my_row < g.M) {
    const int ea = a_ex[g.a_rb0 * OZ_TR + my_row];
    const bool unit = (g.alpha == 1.0 || g.alpha == -1.0) && (g.beta == 0.0 || g.beta == 1.0);
#pragma unroll
    for (int j = 0; j < CPT; ++j) {
      const int64_t col = col0 + half * CPT + j;
      if (col < g.N && !(g.lower_only && my_row < col)) {
        const int sh = ea + b_ex[g.b_rb0 * OZ_TR + col] - 16;
        double v = f2d_scaled(hi[j], sh) + f2d_scaled(lo[j], sh);
        double *dst = Cz + my_row + col * g.ldc;
        if (unit) {
          if (g.alpha < 0.0) v = -v;
          *dst = (g.beta == 0.0) ? v : *dst + v;
        } else {
          *dst = (g.beta == 0.0) ? g.alpha * v : fma(g.alpha, v, g.beta * *dst);
        }
      }
    }
  }
}

void oz_gemm_batched(cudaStream_t s, const OzSplit &A, int64_t a_row0, const OzSplit &B, int64_t b_row0,
                     int64_t M, int64_t N, int64_t kc0, int64_t kc1, int kmode, double alpha,
                     double beta, double *C, int64_t ldc, int64_t sC, bool lower_only, int *err,
                     const int *status, int64_t status_bs, int64_t batch) {
  if (M <= 0 || N <= 0 || batch <= 0) return;
  if (A.S != B.S) throw CudaError{cudaErrorInvalidValue, "oz_gemm: operands split to different slice counts", __LINE__};
  static const bool attr = [] {
    GPGP_CUDA(cudaFuncSetAttribute(oz_gemm_kernel<4>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   OzCfg<4>::SMEM + 1024));
    GPGP_CUDA(cudaFuncSetAttribute(oz_gemm_kernel<5>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   OzCfg<5>::SMEM + 1024));
    return true;
  }();
  (void)attr;
  OzGemmArgs g;
  g.a_sl = A.sl;
  g.a_ex = A.ex;
  g.a_nrb = A.nrb;
  g.a_nkb = A.nkb;
  g.a_rb0 = a_row0 / OZ_TR;
  g.b_sl = B.sl;
  g.b_ex = B.ex;
  g.b_nrb = B.nrb;
  g.b_nkb = B.nkb;
  g.b_rb0 = b_row0 / OZ_TR;
  g.M = M;
  g.N = N;
  g.kc0 = kc0;
  g.kc1 = kc1;
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
  {
    // executed MMA arithmetic of the tiles this launch runs (the kernel's own tile
    // skipping and K ranges), for the per-kernel timer
    const int BN = A.S == 5 ? OzCfg<5>::BN : OzCfg<4>::BN;
    const int prods = A.S == 5 ? 19 : 13;
    const int64_t gx = (M + OZ_BM - 1) / OZ_BM, gy = (N + BN - 1) / BN;
    double fl = 0.0;
    if (tl_kt) {
      for (int64_t bx = 0; bx < gx; ++bx)
        for (int64_t by = 0; by < gy; ++by) {
          const int64_t row0 = bx * OZ_BM, col0 = by * BN;
          if (lower_only && col0 > row0 + OZ_BM - 1) continue;
          const int64_t grow0 = g.a_rb0 * OZ_TR + row0, gcol0 = g.b_rb0 * OZ_TR + col0;
          int64_t k0 = kc0, k1 = kc1;
          if (kmode == 1) k0 = std::max(k0, std::max(grow0, gcol0) / OZ_TK);
          if (kmode == 2) k0 = std::max(k0, gcol0 / OZ_TK);
          if (kmode == 3) k1 = std::min(k1, (grow0 + OZ_BM + OZ_TK - 1) / OZ_TK);
          if (k1 > k0) fl += 2.0 * OZ_BM * BN * OZ_TK * (double)(k1 - k0) * prods;
        }
    }
    KTScope kts(GPGP_KPROF_OZ_GEMM, s, fl * (double)batch);
    if (A.S == 5) {
      dim3 grid((unsigned)gx, (unsigned)gy, (unsigned)batch);
      oz_gemm_kernel<5><<<grid, 256, OzCfg<5>::SMEM + 1024, s>>>(g);
    } else {
      dim3 grid((unsigned)gx, (unsigned)gy, (unsigned)batch);
      oz_gemm_kernel<4><<<grid, 256, OzCfg<4>::SMEM + 1024, s>>>(g);
    }
  }
  GPGP_CHECK_LAUNCH();
}

void oz_gemm(cudaStream_t s, const OzSplit &A, int64_t a_row0, const OzSplit &B, int64_t b_row0,
             int64_t M, int64_t N, int64_t kc0, int64_t kc1, int kmode, double alpha, double beta,
             double *C, int64_t ldc, bool lower_only, int *err, const int *status) {
  oz_gemm_batched(s, A, a_row0, B, b_row0, M, N, kc0, kc1, kmode, alpha, beta, C, ldc, 0, lower_only,
                  err, status, 0, 1);
}


}  // namespace gpgp
