// Covariance functions on the GPU: feature preparation, tile generation,
// fused kernel-matrix x vector, diagonal, and the gradient contraction.
//
// The per-pair formulas restate src/cf.cpp:9-162 (sexp, matern32, matern52,
// nn) and R/cf.R:413-497 (const, lin, periodic, sums and products); inputs
// are prepared as in prepare_inputmat (R/misc.R:17-31).
#include <math.h>

#include <algorithm>
#include <cstring>

#include "bulk.cuh"
#include "common.cuh"
#include "dfloat.cuh"
#include "fp64math.cuh"

namespace gpgp {

std::atomic<int64_t> g_launches{0};
thread_local bool tl_capturing = false;
thread_local KernelTimer *tl_kt = nullptr;

int device_sms() {
  static PerDevice sms;
  return per_device(sms, [] {
    int dev = 0, n = 0;
    GPGP_CUDA(cudaGetDevice(&dev));
    GPGP_CUDA(cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev));
    return n;
  });
}

KTScope::KTScope(int kernel, cudaStream_t st, double flops) : s(st), k(kernel) {
  if (!tl_kt || tl_capturing) return;
  if (cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess) {
    (void)cudaGetLastError();
    a = b = nullptr;
    return;
  }
  cudaEventRecord(a, s);
  tl_kt->flops[k] += flops;
  tl_kt->launches[k] += 1;
}

KTScope::~KTScope() {
  if (!a) return;
  cudaEventRecord(b, s);
  tl_kt->ev.push_back({k, {a, b}});
}

void KernelTimer::collect() {
  for (auto &e : ev) {
    float t = 0.f;
    cudaEventSynchronize(e.second.second);
    cudaEventElapsedTime(&t, e.second.first, e.second.second);
    ms[e.first] += t;
    cudaEventDestroy(e.second.first);
    cudaEventDestroy(e.second.second);
  }
  ev.clear();
}

void KernelTimer::reset() {
  collect();
  for (int i = 0; i < GPGP_NKPROF; ++i) {
    ms[i] = 0;
    flops[i] = 0;
    launches[i] = 0;
  }
}

static const double kPi = 3.14159265358979323846;

gpgp_status build_dev_kernel(const gpgp_kernel *k, int d, DevKernel *dk,
                             std::vector<HostTermPrep> *prep, std::string *err) {
  if (!k || k->nterms < 1 || k->nterms > GPGP_MAX_TERMS || k->ngroups < 1 ||
      k->ngroups > k->nterms || d < 1) {
    *err = "invalid kernel: nterms/ngroups/d out of range";
    return GPGP_EINVAL;
  }
  std::memset(dk, 0, sizeof(*dk));
  prep->clear();
  dk->nterms = k->nterms;
  dk->ngroups = k->ngroups;
  int off = 0, last_group = -1;
  for (int t = 0; t < k->nterms; ++t) {
    const gpgp_cf_term &T = k->term[t];
    if (T.kind < GPGP_CF_CONST || T.kind > GPGP_CF_NN) {
      *err = "invalid kernel: unknown term kind";
      return GPGP_EINVAL;
    }
    if (T.group < 0 || T.group >= k->ngroups || T.group < last_group ||
        (T.group > last_group + 1)) {
      *err = "invalid kernel: groups must be contiguous and numbered 0..ngroups-1";
      return GPGP_EINVAL;
    }
    last_group = T.group;
    HostTermPrep hp;
    std::memset(&hp, 0, sizeof(hp));
    int nv = T.nvars > 0 ? T.nvars : d;
    if (nv > GPGP_MAX_VARS) {
      *err = "invalid kernel: more than GPGP_MAX_VARS input columns in a term";
      return GPGP_EINVAL;
    }
    hp.nv = nv;
    for (int v = 0; v < nv; ++v) {
      int c = T.nvars > 0 ? T.vars[v] : v;
      if (c < 0 || c >= d) {
        *err = "invalid kernel: vars index out of range";
        return GPGP_EINVAL;
      }
      hp.vars[v] = c;
      hp.means[v] = T.means[v];
      hp.scales[v] = T.scales[v];
    }
    hp.periodic = T.periodic ? 1 : 0;
    // cf_periodic never normalises (R/cf.R:173-184, learn_scales.cf_periodic R/cf.R:852)
    hp.normalize = (T.normalize && !T.periodic) ? 1 : 0;
    DevTerm &D = dk->t[t];
    D.kind = T.kind;
    D.group = T.group;
    D.periodic = hp.periodic;
    D.off = off;
    D.nv = nv;
    D.dt = hp.periodic ? 2 * nv : nv;
    D.m2 = T.magn * T.magn;
    if (hp.periodic) {
      if (!(T.period > 0)) {
        *err = "invalid kernel: period must be positive";
        return GPGP_EINVAL;
      }
      hp.w = 2.0 * kPi / T.period;
      D.c2 = hp.w;
    }
    switch (T.kind) {
      case GPGP_CF_SEXP:
        D.c1 = 1.0 / (T.lscale * T.lscale);
        break;
      case GPGP_CF_MATERN32:
        D.c1 = sqrt(3.0) / T.lscale;
        break;
      case GPGP_CF_MATERN52:
        D.c1 = sqrt(5.0) / T.lscale;
        break;
      case GPGP_CF_NN:
        D.c1 = T.sigma0 * T.sigma0 * T.sigma * T.sigma;
        if (!hp.periodic) D.c2 = T.sigma * T.sigma;
        break;
      default:
        break;
    }
    if (T.kind == GPGP_CF_NN && hp.periodic) {
      *err = "periodic wrapper around cf_nn is not supported";
      return GPGP_EUNSUPPORTED;
    }
    off += hp.periodic ? 3 * nv : nv;
    prep->push_back(hp);
  }
  if (last_group != k->ngroups - 1) {
    *err = "invalid kernel: ngroups does not match the groups used";
    return GPGP_EINVAL;
  }
  if (off > 64) {
    *err = "invalid kernel: more than 64 feature columns in total";
    return GPGP_EINVAL;
  }
  dk->nfeat = off;
  return GPGP_OK;
}

// ---------------------------------------------------------------------------
// feature preparation
// ---------------------------------------------------------------------------
struct FeatCol {
  int src;   // input column
  int mode;  // 0 raw, 1 normalised, 2 sin(w x), 3 cos(w x)
  double mean, scale, w;
};
struct FeatTable {
  int ncol;
  FeatCol c[64];
};

__global__ void prep_features_kernel(FeatTable tab, const double *__restrict__ x, int64_t n,
                                     int64_t ldx, double *__restrict__ F, int64_t ldf) {
  int col = blockIdx.y;
  const FeatCol fc = tab.c[col];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double v = x[i + fc.src * ldx];
    double o;
    if (fc.mode == 1)
      o = (v - fc.mean) / fc.scale;
    else if (fc.mode == 2)
      o = sin(fc.w * v);
    else if (fc.mode == 3)
      o = cos(fc.w * v);
    else
      o = v;
    F[i + col * ldf] = o;
  }
}

void prep_features(cudaStream_t s, const DevKernel &dk, const std::vector<HostTermPrep> &prep,
                   const double *x, int64_t n, int64_t ldx, double *F, int64_t ldf) {
  FeatTable tab;
  std::memset(&tab, 0, sizeof(tab));
  int c = 0;
  for (int t = 0; t < dk.nterms; ++t) {
    const HostTermPrep &hp = prep[t];
    if (hp.periodic) {
      // cbind(sin(2*pi/period * x), cos(2*pi/period * x)) (R/cf.R:482-483), then raw
      // columns for the period derivative
      for (int v = 0; v < hp.nv; ++v) tab.c[c++] = FeatCol{hp.vars[v], 2, 0.0, 1.0, hp.w};
      for (int v = 0; v < hp.nv; ++v) tab.c[c++] = FeatCol{hp.vars[v], 3, 0.0, 1.0, hp.w};
      for (int v = 0; v < hp.nv; ++v) tab.c[c++] = FeatCol{hp.vars[v], 0, 0.0, 1.0, 0.0};
    } else {
      for (int v = 0; v < hp.nv; ++v)
        tab.c[c++] = FeatCol{hp.vars[v], hp.normalize ? 1 : 0, hp.means[v], hp.scales[v], 0.0};
    }
  }
  tab.ncol = c;
  if (n == 0 || c == 0) return;
  int64_t bx = std::min<int64_t>((n + 255) / 256, 4096);
  dim3 grid((unsigned)bx, (unsigned)c);
  prep_features_kernel<<<grid, 256, 0, s>>>(tab, x, n, ldx, F, ldf);
  GPGP_CHECK_LAUNCH();
}

// ---------------------------------------------------------------------------
// per-pair evaluation
// ---------------------------------------------------------------------------
// fi / fj point at the term's first feature of points i and j (stride 1).
__device__ __forceinline__ double term_value(const DevTerm &T, const double *fi,
                                             const double *fj) {
  switch (T.kind) {
    case GPGP_CF_CONST:
      return T.m2;
    case GPGP_CF_LIN: {
      double dot = 0.0;
      for (int c = 0; c < T.dt; ++c) dot += fi[c] * fj[c];
      return T.m2 * dot;
    }
    case GPGP_CF_NN: {
      double a = 0.0, b = 0.0, cc = 0.0;
      for (int c = 0; c < T.dt; ++c) {
        a += fi[c] * fj[c];
        b += fi[c] * fi[c];
        cc += fj[c] * fj[c];
      }
      a = T.c1 + T.c2 * a;
      b = T.c1 + T.c2 * b;
      cc = T.c1 + T.c2 * cc;
      return T.m2 * (2.0 / 3.14159265358979323846) * asin(2.0 * a / sqrt((1.0 + 2.0 * b) * (1.0 + 2.0 * cc)));
    }
    default: {
      double r2 = 0.0;
      for (int c = 0; c < T.dt; ++c) {
        double df = fi[c] - fj[c];
        r2 += df * df;
      }
      if (T.kind == GPGP_CF_SEXP) return T.m2 * exp_fast(-0.5 * r2 * T.c1);
      double a = T.c1 * sqrt_fast(r2);
      if (T.kind == GPGP_CF_MATERN32) return T.m2 * (1.0 + a) * exp_fast(-a);
      return T.m2 * (1.0 + a + a * a * (1.0 / 3.0)) * exp_fast(-a);
    }
  }
}

// K(i, j) = sum over selected groups of the product of the group's terms.
__device__ __forceinline__ double kernel_value(const DevKernel &dk, uint32_t gmask,
                                               const double *fi, const double *fj) {
  double sum = 0.0, prod = 1.0;
  int g = dk.t[0].group;
  for (int t = 0; t < dk.nterms; ++t) {
    const DevTerm &T = dk.t[t];
    if (T.group != g) {
      if (gmask & (1u << g)) sum += prod;
      prod = 1.0;
      g = T.group;
    }
    prod *= term_value(T, fi + T.off, fj + T.off);
  }
  if (gmask & (1u << g)) sum += prod;
  return sum;
}

// ---------------------------------------------------------------------------
// tile generator
// ---------------------------------------------------------------------------
constexpr int CT = 64;  // tile edge

__device__ __forceinline__ void tri_index(int64_t idx, int64_t *bi, int64_t *bj) {
  // idx -> (bi, bj) with bi >= bj, row-major over the lower triangle of tiles
  int64_t b = (int64_t)((sqrt(8.0 * (double)idx + 1.0) - 1.0) * 0.5);
  while (b * (b + 1) / 2 > idx) --b;
  while ((b + 1) * (b + 2) / 2 <= idx) ++b;
  *bi = b;
  *bj = idx - b * (b + 1) / 2;
}

__device__ __forceinline__ void load_feats(double *dst, int lds, const double *F, int64_t ld,
                                           int64_t row0, int64_t n, int nfeat) {
  for (int idx = threadIdx.x; idx < CT * nfeat; idx += blockDim.x) {
    int r = idx % CT, c = idx / CT;
    int64_t row = row0 + r;
    dst[r * lds + c] = row < n ? F[row + c * ld] : 0.0;
  }
}

template <int TT>
__device__ __forceinline__ void load_feats_t(double *dst, int lds, const double *F, int64_t ld, int64_t row0,
                                             int64_t n, int nfeat) {
  for (int idx = threadIdx.x; idx < TT * nfeat; idx += blockDim.x) {
    int r = idx % TT, c = idx / TT;
    int64_t row = row0 + r;
    dst[r * lds + c] = row < n ? F[row + c * ld] : 0.0;
  }
}

// Stages rows [i0, i0 + ri) of the nf feature columns of F1 (leading dimension ld1)
// and, when two, rows [j0, j0 + rj) of F2's into raw (column-major, TT rows per
// column: raw[c TT + r], then raw[(nf + c) TT + r]) with the TMA unit: thread 0
// issues one cp.async.bulk per column completing on the mbarrier bar and waits for
// them (bounded). Every copy must start on a 16-byte boundary and move a multiple
// of 16 bytes (the caller checks). All threads call it; it ends with a barrier and
// returns false for the whole block when the wait ran out (*err |= 1), after
// letting the copies land.
template <int TT>
__device__ __forceinline__ bool stage_features_bulk(double *raw, uint64_t *bar, const double *F1, int64_t ld1,
                                                    int64_t i0, int64_t ri, const double *F2, int64_t ld2,
                                                    int64_t j0, int64_t rj, bool two, int nf, int *err) {
  volatile int *landed = reinterpret_cast<volatile int *>(bar + 1);
  if (threadIdx.x == 0) {
    const uint32_t b0 = smem_u32(bar);
    mbar_init(b0, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    mbar_expect_tx(b0, (uint32_t)((ri + (two ? rj : 0)) * nf * sizeof(double)));
    for (int c = 0; c < nf; ++c) {
      bulk_g2s(smem_u32(raw + c * TT), F1 + i0 + c * ld1, (uint32_t)(ri * sizeof(double)), b0);
      if (two) bulk_g2s(smem_u32(raw + (nf + c) * TT), F2 + j0 + c * ld2, (uint32_t)(rj * sizeof(double)), b0);
    }
    const bool ok = mbar_wait_bounded(b0, 0);
    if (!ok) {
      atomicOr(err, 1);
      mbar_wait_bounded(b0, 0);  // let the copies land before the block's shared memory goes
    }
    *landed = ok ? 1 : 0;
  }
  __syncthreads();
  return *landed != 0;
}

// TMA staging is possible when every copy of a TT-row tile of F (leading
// dimension ld, n rows) starts on a 16-byte boundary and moves a multiple of 16 bytes.
inline bool bulk_ok(const double *F, int64_t ld, int64_t n) {
  return F && ((uintptr_t)F & 15) == 0 && ld % 2 == 0 && n % 2 == 0;
}

// TT x TT tiles (TT = 64; 16 for small matrices, so that their tiles spread over
// more SMs); 256 / TT column groups of threads.
template <int TT>
__global__ void __launch_bounds__(256) cov_tile_kernel(DevKernel dk, uint32_t gmask, const double *__restrict__ F1, int64_t ld1, int64_t n1,
                                const double *__restrict__ F2, int64_t ld2, int64_t n2,
                                double *__restrict__ out, int64_t ldo, int mode, int sym,
                                int mirror, double jitter, const double *__restrict__ scale, int *err) {
  extern __shared__ __align__(16) double sm[];
  const int nf = dk.nfeat;
  const int lds = (nf | 1);
  // err: TMA staging of the feature rows (raw, the mbarrier), else plain loads
  double *raw = sm;
  uint64_t *bar = reinterpret_cast<uint64_t *>(raw + (err ? 2 * nf * TT : 0));
  double *Fi = reinterpret_cast<double *>(bar + (err ? 2 : 0));
  double *Fj = Fi + TT * lds;
  double *Tt = Fi + 2 * TT * lds;  // TT x (TT+1) staging for the mirrored write
  int64_t bi, bj;
  if (sym)
    tri_index(blockIdx.x, &bi, &bj);
  else {
    bi = blockIdx.x;
    bj = blockIdx.y;
  }
  const int64_t i0 = bi * TT, j0 = bj * TT;
  constexpr int CG = 256 / TT;
  if (err) {
    const int64_t ri = n1 - i0 < TT ? n1 - i0 : TT, rj = n2 - j0 < TT ? n2 - j0 : TT;
    if (!stage_features_bulk<TT>(raw, bar, F1, ld1, i0, ri, F2, ld2, j0, rj, true, nf, err)) return;
    for (int idx = threadIdx.x; idx < TT * nf; idx += blockDim.x) {
      const int r = idx % TT, c = idx / TT;
      Fi[r * lds + c] = r < ri ? raw[c * TT + r] : 0.0;
      Fj[r * lds + c] = r < rj ? raw[(nf + c) * TT + r] : 0.0;
    }
  } else {
    load_feats_t<TT>(Fi, lds, F1, ld1, i0, n1, nf);
    load_feats_t<TT>(Fj, lds, F2, ld2, j0, n2, nf);
  }
  __syncthreads();
  const int r = threadIdx.x % TT;
  const int cb = threadIdx.x / TT;
  const int64_t i = i0 + r;
  const double si = (mode == COV_ROWSCALE && i < n1) ? scale[i] : 1.0;
  const bool do_mirror = sym && mirror && bi != bj;
#pragma unroll 1
  for (int q = 0; q < TT / CG; ++q) {
    const int c = cb + CG * q;
    const int64_t j = j0 + c;
    double v = 0.0;
    if (i < n1 && j < n2) {
      v = kernel_value(dk, gmask, Fi + r * lds, Fj + c * lds);
      if (sym && i == j) v += jitter;
      if (mode == COV_ROWSCALE) v = si * v;
      out[i + j * ldo] = v;
    }
    if (do_mirror) Tt[c * (TT + 1) + r] = v;
  }
  if (do_mirror) {
    __syncthreads();
    // transposed tile: rows j0.., cols i0..
#pragma unroll 1
    for (int q = 0; q < TT / CG; ++q) {
      const int rr = threadIdx.x % TT;  // row inside the transposed tile (j index)
      const int cc = threadIdx.x / TT + CG * q;  // col (i index)
      const int64_t jj = j0 + rr, ii = i0 + cc;
      if (jj < n2 && ii < n1) out[jj + ii * ldo] = Tt[rr * (TT + 1) + cc];
    }
  }
}

void cov_matrix(cudaStream_t s, const DevKernel &dk, uint32_t group_mask, const double *F1,
                int64_t ld1, int64_t n1, const double *F2, int64_t ld2, int64_t n2, double *out,
                int64_t ldo, int mode, int sym, int mirror, double jitter, const double *scale, int *err) {
  if (n1 == 0 || n2 == 0) return;
  const int lds = (dk.nfeat | 1);
  // TMA staging when asked for (err) and every copy is aligned
  if (!(err && dk.nfeat <= 64 && bulk_ok(F1, ld1, n1) && bulk_ok(F2, ld2, n2))) err = nullptr;
  const size_t stage = err ? (size_t)2 * dk.nfeat * sizeof(double) : 0;  // per tile row, plus the mbarrier
  size_t smem = (size_t)(2 * CT * lds + CT * (CT + 1)) * sizeof(double) + (err ? CT * stage + 16 : 0);
  static PerDevice attr;
  per_device(attr, [] {
    GPGP_CUDA(cudaFuncSetAttribute(cov_tile_kernel<CT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   2 * CT * 65 * 8 + CT * (CT + 1) * 8 + 2 * 64 * CT * 8 + 16));
    return 1;
  });
  int64_t T1 = (n1 + CT - 1) / CT, T2 = (n2 + CT - 1) / CT;
  // fewer 64-tiles than SMs: 16-tiles (the evaluation is FP64-bound per SM)
  const bool small = (sym ? T1 * (T1 + 1) / 2 : T1 * T2) < device_sms();
  if (small) {
    constexpr int ST = 16;
    smem = (size_t)(2 * ST * lds + ST * (ST + 1)) * sizeof(double) + (err ? ST * stage + 16 : 0);
    T1 = (n1 + ST - 1) / ST;
    T2 = (n2 + ST - 1) / ST;
    if (sym)
      cov_tile_kernel<ST><<<(unsigned)(T1 * (T1 + 1) / 2), 256, smem, s>>>(dk, group_mask, F1, ld1, n1, F2, ld2, n2,
                                                                            out, ldo, mode, 1, mirror, jitter, scale,
                                                                            err);
    else
      cov_tile_kernel<ST><<<dim3((unsigned)T1, (unsigned)T2), 256, smem, s>>>(
          dk, group_mask, F1, ld1, n1, F2, ld2, n2, out, ldo, mode, 0, 0, 0.0, scale, err);
  } else if (sym) {
    int64_t nt = T1 * (T1 + 1) / 2;
    cov_tile_kernel<CT><<<(unsigned)nt, 256, smem, s>>>(dk, group_mask, F1, ld1, n1, F2, ld2, n2, out,
                                                        ldo, mode, 1, mirror, jitter, scale, err);
  } else {
    dim3 grid((unsigned)T1, (unsigned)T2);
    cov_tile_kernel<CT><<<grid, 256, smem, s>>>(dk, group_mask, F1, ld1, n1, F2, ld2, n2, out, ldo,
                                                mode, 0, 0, 0.0, scale, err);
  }
  GPGP_CHECK_LAUNCH();
}

// ---------------------------------------------------------------------------
// diagonal
// ---------------------------------------------------------------------------
__global__ void cov_diag_kernel(DevKernel dk, uint32_t gmask, const double *__restrict__ F1,
                                int64_t ld1, const double *__restrict__ F2, int64_t ld2,
                                int64_t n, double *__restrict__ out) {
  double fi[64], fj[64];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    for (int c = 0; c < dk.nfeat; ++c) {
      fi[c] = F1[i + c * ld1];
      fj[c] = F2[i + c * ld2];
    }
    out[i] = kernel_value(dk, gmask, fi, fj);
  }
}

void cov_diag(cudaStream_t s, const DevKernel &dk, uint32_t group_mask, const double *F1,
              int64_t ld1, const double *F2, int64_t ld2, int64_t n, double *out) {
  if (n == 0) return;
  int64_t b = std::min<int64_t>((n + 127) / 128, 8192);
  cov_diag_kernel<<<(unsigned)b, 128, 0, s>>>(dk, group_mask, F1, ld1, F2, ld2, n, out);
  GPGP_CHECK_LAUNCH();
}

// ---------------------------------------------------------------------------
// fused K x v
// ---------------------------------------------------------------------------
// Block (x, y) takes rows [x CT, (x+1) CT) of x1 and the y-th of gridDim.y equal
// ranges of x2 tiles; with one range it writes out, otherwise its partial sums go to
// out + y n1 and a second kernel adds the ranges in order.
__global__ void __launch_bounds__(256) cov_matvec_kernel(DevKernel dk, uint32_t gmask, const double *__restrict__ F1, int64_t ld1, int64_t n1,
                                  const double *__restrict__ F2, int64_t ld2, int64_t n2,
                                  const double *__restrict__ v, double *__restrict__ out,
                                  int64_t tiles_per_range) {
  extern __shared__ double sm[];
  const int nf = dk.nfeat;
  const int lds = (nf | 1);
  double *Fi = sm;
  double *Fj = sm + CT * lds;
  double *vj = sm + 2 * CT * lds;
  double *red = vj + CT;  // 4 x CT partials
  const int64_t i0 = (int64_t)blockIdx.x * CT;
  out += (int64_t)blockIdx.y * n1;
  load_feats(Fi, lds, F1, ld1, i0, n1, nf);
  const int r = threadIdx.x % CT;
  const int cb = threadIdx.x / CT;
  double acc = 0.0;
  const int64_t jbeg = (int64_t)blockIdx.y * tiles_per_range * CT;
  const int64_t jlim = jbeg + tiles_per_range * CT;
  const int64_t jend = jlim < n2 ? jlim : n2;
  for (int64_t j0 = jbeg; j0 < jend; j0 += CT) {
    __syncthreads();
    load_feats(Fj, lds, F2, ld2, j0, n2, nf);
    if (threadIdx.x < CT) vj[threadIdx.x] = (j0 + threadIdx.x < n2) ? v[j0 + threadIdx.x] : 0.0;
    __syncthreads();
    if (i0 + r < n1) {
#pragma unroll 1
      for (int q = 0; q < CT / 4; ++q) {
        const int c = cb * (CT / 4) + q;
        if (j0 + c < n2) acc += kernel_value(dk, gmask, Fi + r * lds, Fj + c * lds) * vj[c];
      }
    }
  }
  red[cb * CT + r] = acc;
  __syncthreads();
  if (threadIdx.x < CT && i0 + threadIdx.x < n1) {
    double t = red[threadIdx.x];
    for (int k = 1; k < 4; ++k) t += red[k * CT + threadIdx.x];
    out[i0 + threadIdx.x] = t;
  }
}

// out[i] = sum over the ranges r (in order) of part[r n1 + i]
__global__ void sum_ranges_kernel(const double *__restrict__ part, int64_t nr, int64_t n1,
                                  double *__restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n1) return;
  double t = part[i];
  for (int64_t r = 1; r < nr; ++r) t += part[r * n1 + i];
  out[i] = t;
}

void cov_matvec(cudaStream_t s, const DevKernel &dk, uint32_t group_mask, const double *F1,
                int64_t ld1, int64_t n1, const double *F2, int64_t ld2, int64_t n2,
                const double *v, double *out) {
  if (n1 == 0) return;
  const int lds = (dk.nfeat | 1);
  size_t smem = (size_t)(2 * CT * lds + CT + 4 * CT) * sizeof(double);
  static PerDevice attr;
  per_device(attr, [] {
    GPGP_CUDA(cudaFuncSetAttribute(cov_matvec_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (2 * CT * 65 + 5 * CT) * 8));
    return 1;
  });
  const int64_t T1 = (n1 + CT - 1) / CT, T2 = std::max<int64_t>(1, (n2 + CT - 1) / CT);
  // enough blocks for two per SM: split the x2 tiles into equal ranges
  const int64_t want = std::max<int64_t>(1, (2 * device_sms() + T1 - 1) / T1);
  const int64_t tpr = (T2 + std::min(want, T2) - 1) / std::min(want, T2);
  const int64_t nrange = (T2 + tpr - 1) / tpr;
  if (nrange == 1) {
    cov_matvec_kernel<<<dim3((unsigned)T1, 1), 256, smem, s>>>(dk, group_mask, F1, ld1, n1, F2, ld2, n2, v, out,
                                                               tpr);
    GPGP_CHECK_LAUNCH();
    return;
  }
  double *part = nullptr;
  GPGP_CUDA(cudaMallocAsync((void **)&part, (size_t)nrange * n1 * sizeof(double), s));
  cov_matvec_kernel<<<dim3((unsigned)T1, (unsigned)nrange), 256, smem, s>>>(dk, group_mask, F1, ld1, n1, F2, ld2,
                                                                            n2, v, part, tpr);
  GPGP_CHECK_LAUNCH();
  sum_ranges_kernel<<<(unsigned)((n1 + 255) / 256), 256, 0, s>>>(part, nrange, n1, out);
  GPGP_CHECK_LAUNCH();
  GPGP_CUDA(cudaFreeAsync(part, s));
}

// ---------------------------------------------------------------------------
// gradient contraction
// ---------------------------------------------------------------------------
// Derivatives of one term with respect to the log of its parameters:
// slot 0 lscale, 1 magn, 2 sigma0, 3 sigma, 4 period. fi/fj point at the
// term's features; for periodic terms fi[2*nv + k] are the raw inputs.
__device__ __forceinline__ double term_value_grad(const DevTerm &T, const double *fi,
                                                  const double *fj, double dv[5]) {
  dv[0] = dv[1] = dv[2] = dv[3] = dv[4] = 0.0;
  double k;
  switch (T.kind) {
    case GPGP_CF_CONST:
      k = T.m2;
      dv[1] = 2.0 * k;
      return k;
    case GPGP_CF_LIN: {
      double dot = 0.0;
      for (int c = 0; c < T.dt; ++c) dot += fi[c] * fj[c];
      k = T.m2 * dot;
      dv[1] = 2.0 * k;
      if (T.periodic) {
        // sum_k cos(w (x_k - y_k)) -> d/dlog p = sum_k w d_k sin(w d_k)
        double acc = 0.0;
        for (int c = 0; c < T.nv; ++c) {
          double dd = fi[2 * T.nv + c] - fj[2 * T.nv + c];
          double sn = fi[c] * fj[T.nv + c] - fi[T.nv + c] * fj[c];  // sin(w dd)
          acc += T.c2 * dd * sn;
        }
        dv[4] = T.m2 * acc;
      }
      return k;
    }
    case GPGP_CF_NN: {
      double a = 0.0, b = 0.0, cc = 0.0;
      for (int c = 0; c < T.dt; ++c) {
        a += fi[c] * fj[c];
        b += fi[c] * fi[c];
        cc += fj[c] * fj[c];
      }
      a = T.c1 + T.c2 * a;
      b = T.c1 + T.c2 * b;
      cc = T.c1 + T.c2 * cc;
      const double q = sqrt((1.0 + 2.0 * b) * (1.0 + 2.0 * cc));
      const double u = 2.0 * a / q;
      k = T.m2 * (2.0 / 3.14159265358979323846) * asin(u);
      const double dk_du = T.m2 * (2.0 / 3.14159265358979323846) / sqrt(1.0 - u * u);
      // d/dlog sigma0: da = db = dc = 2 s0
      const double ds0 = 2.0 * T.c1;
      double du = 2.0 * ds0 / q - u * (ds0 / (1.0 + 2.0 * b) + ds0 / (1.0 + 2.0 * cc));
      dv[2] = dk_du * du;
      // d/dlog sigma: da = 2a, db = 2b, dc = 2c
      du = 4.0 * a / q - u * (2.0 * b / (1.0 + 2.0 * b) + 2.0 * cc / (1.0 + 2.0 * cc));
      dv[3] = dk_du * du;
      dv[1] = 2.0 * k;
      return k;
    }
    default: {
      double r2 = 0.0;
      for (int c = 0; c < T.dt; ++c) {
        double df = fi[c] - fj[c];
        r2 += df * df;
      }
      double dk_dr2;
      if (T.kind == GPGP_CF_SEXP) {
        k = T.m2 * exp_fast(-0.5 * r2 * T.c1);
        dv[0] = k * r2 * T.c1;
        dk_dr2 = -0.5 * T.c1 * k;
      } else {
        const double a = T.c1 * sqrt_fast(r2);
        const double e = exp_fast(-a);
        if (T.kind == GPGP_CF_MATERN32) {
          k = T.m2 * (1.0 + a) * e;
          dv[0] = T.m2 * a * a * e;
          dk_dr2 = -0.5 * T.m2 * T.c1 * T.c1 * e;
        } else {
          k = T.m2 * (1.0 + a + a * a * (1.0 / 3.0)) * e;
          dv[0] = T.m2 * a * a * (1.0 + a) * (1.0 / 3.0) * e;
          dk_dr2 = -T.m2 * T.c1 * T.c1 * (1.0 / 6.0) * (1.0 + a) * e;
        }
      }
      dv[1] = 2.0 * k;
      if (T.periodic) {
        // r2 = sum_k 2 - 2 cos(w d_k); d r2 / dlog p = -w sum_k 2 d_k sin(w d_k)
        double acc = 0.0;
        for (int c = 0; c < T.nv; ++c) {
          double dd = fi[2 * T.nv + c] - fj[2 * T.nv + c];
          double sn = fi[c] * fj[T.nv + c] - fi[T.nv + c] * fj[c];
          acc += 2.0 * dd * sn;
        }
        dv[4] = dk_dr2 * (-T.c2 * acc);
      }
      return k;
    }
  }
}

// parameter slots that term_value_grad can set for a term (bit p: slot p)
__host__ __device__ __forceinline__ int term_param_mask(const DevTerm &T) {
  switch (T.kind) {
    case GPGP_CF_CONST:
      return 2;
    case GPGP_CF_LIN:
      return 2 | (T.periodic ? 16 : 0);
    case GPGP_CF_NN:
      return 14;
    default:
      return 3 | (T.periodic ? 16 : 0);
  }
}

constexpr int GT = 64;

// NT > 0: a kernel of exactly NT terms, loops unrolled so that the accumulators
// stay in registers; NT == 0: any number of terms (dk.nterms).
template <int NT>
__global__ void __launch_bounds__(256) cov_grad_kernel(DevKernel dk, const double *__restrict__ F, int64_t ldf, int64_t n,
                                const double *__restrict__ W, int64_t ldw,
                                double *__restrict__ part) {
  extern __shared__ double sm[];
  constexpr int MT = NT > 0 ? NT : GPGP_MAX_TERMS;
  const int nterms = NT > 0 ? NT : dk.nterms;
  const int nf = dk.nfeat;
  const int lds = (nf | 1);
  double *Fi = sm;
  double *Fj = sm + GT * lds;
  double *red = sm + 2 * GT * lds;  // 256 doubles
  int64_t bi, bj;
  tri_index(blockIdx.x, &bi, &bj);
  const int64_t i0 = bi * GT, j0 = bj * GT;
  load_feats(Fi, lds, F, ldf, i0, n, nf);
  load_feats(Fj, lds, F, ldf, j0, n, nf);
  __syncthreads();
  const int np = nterms * GPGP_TERM_NPARAM;
  double acc[MT * GPGP_TERM_NPARAM];
#pragma unroll
  for (int p = 0; p < MT * GPGP_TERM_NPARAM; ++p) acc[p] = 0.0;
  int pmask[MT];
#pragma unroll
  for (int t = 0; t < MT; ++t) pmask[t] = t < nterms ? term_param_mask(dk.t[t]) : 0;
  const int r = threadIdx.x % GT;
  const int cb = threadIdx.x / GT;
  const int64_t i = i0 + r;
  double kv[MT];
  double dv[MT][GPGP_TERM_NPARAM];
#pragma unroll 1
  for (int q = 0; q < GT / 4; ++q) {
    const int c = cb + 4 * q;
    const int64_t j = j0 + c;
    if (i >= n || j >= n || j > i) continue;
    const double w = W[i + j * ldw] * (i == j ? 1.0 : 2.0);
#pragma unroll
    for (int t = 0; t < MT; ++t)
      if (t < nterms)
        kv[t] = term_value_grad(dk.t[t], Fi + r * lds + dk.t[t].off, Fj + c * lds + dk.t[t].off, dv[t]);
#pragma unroll
    for (int t = 0; t < MT; ++t) {
      if (t >= nterms) break;
      double others = 1.0;
#pragma unroll
      for (int u = 0; u < MT; ++u)
        if (u < nterms && u != t && dk.t[u].group == dk.t[t].group) others *= kv[u];
      const double f = w * others;
#pragma unroll
      for (int p = 0; p < GPGP_TERM_NPARAM; ++p)
        if (pmask[t] & (1 << p)) acc[t * GPGP_TERM_NPARAM + p] = fma(f, dv[t][p], acc[t * GPGP_TERM_NPARAM + p]);
    }
  }
  // block reduction per parameter, fixed order
#pragma unroll
  for (int p = 0; p < MT * GPGP_TERM_NPARAM; ++p) {
    if (p >= np) break;
    red[threadIdx.x] = acc[p];
    __syncthreads();
    for (int st = 128; st > 0; st >>= 1) {
      if (threadIdx.x < st) red[threadIdx.x] += red[threadIdx.x + st];
      __syncthreads();
    }
    if (threadIdx.x == 0) part[(int64_t)blockIdx.x * np + p] = red[0];
    __syncthreads();
  }
}

__global__ void reduce_partials_kernel(const double *__restrict__ part, int64_t nblocks, int np,
                                       double *__restrict__ g) {
  // one warp per parameter, fixed summation order
  __shared__ double red[256];
  for (int p = 0; p < np; ++p) {
    double acc = 0.0;
    for (int64_t b = threadIdx.x; b < nblocks; b += blockDim.x) acc += part[b * np + p];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int st = 128; st > 0; st >>= 1) {
      if (threadIdx.x < st) red[threadIdx.x] += red[threadIdx.x + st];
      __syncthreads();
    }
    if (threadIdx.x == 0) g[p] = red[0];
    __syncthreads();
  }
}

int64_t cov_grad_partials(int64_t n) {
  int64_t T = (n + GT - 1) / GT;
  return T * (T + 1) / 2 * GPGP_MAX_TERMS * GPGP_TERM_NPARAM;
}

gpgp_status cov_grad_contract(cudaStream_t s, const DevKernel &dk, const double *F, int64_t ldf,
                              int64_t n, const double *W, int64_t ldw, double *part, double *g) {
  const int lds = (dk.nfeat | 1);
  size_t smem = (size_t)(2 * GT * lds + 256) * sizeof(double);
  static PerDevice attr;
  per_device(attr, [] {
    const int mx = (2 * GT * 65 + 256) * 8;
    GPGP_CUDA(cudaFuncSetAttribute(cov_grad_kernel<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx));
    GPGP_CUDA(cudaFuncSetAttribute(cov_grad_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx));
    GPGP_CUDA(cudaFuncSetAttribute(cov_grad_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx));
    GPGP_CUDA(cudaFuncSetAttribute(cov_grad_kernel<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx));
    return 1;
  });
  int64_t T = (n + GT - 1) / GT;
  int64_t nt = T * (T + 1) / 2;
  switch (dk.nterms) {
    case 1:
      cov_grad_kernel<1><<<(unsigned)nt, 256, smem, s>>>(dk, F, ldf, n, W, ldw, part);
      break;
    case 2:
      cov_grad_kernel<2><<<(unsigned)nt, 256, smem, s>>>(dk, F, ldf, n, W, ldw, part);
      break;
    case 3:
      cov_grad_kernel<3><<<(unsigned)nt, 256, smem, s>>>(dk, F, ldf, n, W, ldw, part);
      break;
    default:
      cov_grad_kernel<0><<<(unsigned)nt, 256, smem, s>>>(dk, F, ldf, n, W, ldw, part);
  }
  GPGP_CHECK_LAUNCH();
  reduce_partials_kernel<<<1, 256, 0, s>>>(part, nt, dk.nterms * GPGP_TERM_NPARAM, g);
  GPGP_CHECK_LAUNCH();
  return GPGP_OK;
}

// ---------------------------------------------------------------------------
// K together with its derivative matrices (the energy gradient follows the fit)
// ---------------------------------------------------------------------------
// The gradient contraction above regenerates every derivative tile from the
// features after the factorisation: the same distances, square roots and
// exponentials as the covariance, on the FP64 pipe, a second time. When the
// gradient is known to follow the fit, the covariance pass writes the
// derivative matrices beside K instead (the extra FP64 work per pair is a few
// multiplications), and the contraction becomes a stream over W and them.
//
// Every magnitude slot of a product group has the derivative 2 x (the group's
// value), so one matrix per group serves all of them; a group made only of
// cf_const terms has a constant value and needs none. Every other active slot
// (lscale, sigma0, sigma, period) gets its own matrix: (the product of the
// group's other terms) x (the term's derivative).
bool plan_grad_store(const DevKernel &dk, GradPlan *pl) {
  std::memset(pl, 0, sizeof(*pl));
  bool allconst[GPGP_MAX_TERMS];
  double constprod[GPGP_MAX_TERMS];
  int gmat[GPGP_MAX_TERMS];
  for (int g = 0; g < GPGP_MAX_TERMS; ++g) {
    allconst[g] = true;
    constprod[g] = 1.0;
    gmat[g] = -1;
  }
  for (int t = 0; t < dk.nterms; ++t) {
    if (dk.t[t].kind != GPGP_CF_CONST) allconst[dk.t[t].group] = false;
    constprod[dk.t[t].group] *= dk.t[t].m2;
  }
  for (int t = 0; t < dk.nterms; ++t) {
    const DevTerm &T = dk.t[t];
    const int mask = term_param_mask(T);
    for (int p = 0; p < GPGP_TERM_NPARAM; ++p) {
      const int idx = t * GPGP_TERM_NPARAM + p;
      pl->slot_mat[idx] = -2;
      pl->slot_scale[idx] = 0.0;
      if (!(mask & (1 << p))) continue;
      if (p == 1) {
        if (allconst[T.group]) {
          pl->slot_mat[idx] = -1;  // constant 2 x (product of the group's m^2)
          pl->slot_scale[idx] = 2.0 * constprod[T.group];
          continue;
        }
        if (gmat[T.group] < 0) {
          if (pl->m.nmat == GPGP_GRAD_MAXMAT) return false;
          gmat[T.group] = pl->m.nmat;
          pl->m.kind[pl->m.nmat] = 0;
          pl->m.a[pl->m.nmat] = T.group;
          pl->m.grp[pl->m.nmat] = T.group;
          pl->m.b[pl->m.nmat] = 0;
          ++pl->m.nmat;
        }
        pl->slot_mat[idx] = gmat[T.group];
        pl->slot_scale[idx] = 2.0;
      } else {
        if (pl->m.nmat == GPGP_GRAD_MAXMAT) return false;
        pl->m.kind[pl->m.nmat] = 1;
        pl->m.a[pl->m.nmat] = t;
        pl->m.grp[pl->m.nmat] = T.group;
        pl->m.b[pl->m.nmat] = p;
        pl->slot_mat[idx] = pl->m.nmat++;
        pl->slot_scale[idx] = 1.0;
      }
    }
  }
  return true;
}

// Lower 64 x 64 tiles of K (mirrored, jitter on the diagonal; the same values
// as cov_tile_kernel) and, for entries i >= j, the planned derivative matrices
// D + q dstride (leading dimension ldd).
template <int NT>
__global__ void __launch_bounds__(256) cov_tile_grad_kernel(DevKernel dk, GradMats gm, const double *__restrict__ F,
                                                            int64_t ldf, int64_t n, double *__restrict__ K,
                                                            int64_t ldk, double jitter, double *__restrict__ D,
                                                            int64_t ldd, int64_t dstride, int *err) {
  extern __shared__ __align__(16) double sm[];
  constexpr int MT = NT > 0 ? NT : GPGP_MAX_TERMS;
  const int nterms = NT > 0 ? NT : dk.nterms;
  const int nf = dk.nfeat;
  const int lds = (nf | 1);
  // err: TMA staging of the feature rows (raw, the mbarrier), else plain loads
  double *raw = sm;
  uint64_t *bar = reinterpret_cast<uint64_t *>(raw + (err ? 2 * nf * CT : 0));
  double *Fi = reinterpret_cast<double *>(bar + (err ? 2 : 0));
  double *Fj = Fi + CT * lds;
  double *Tt = Fi + 2 * CT * lds;  // CT x (CT+1) staging for the mirrored write
  int64_t bi, bj;
  tri_index(blockIdx.x, &bi, &bj);
  const int64_t i0 = bi * CT, j0 = bj * CT;
  if (err) {
    const int64_t ri = n - i0 < CT ? n - i0 : CT, rj = n - j0 < CT ? n - j0 : CT;
    if (!stage_features_bulk<CT>(raw, bar, F, ldf, i0, ri, F, ldf, j0, rj, true, nf, err)) return;
    for (int idx = threadIdx.x; idx < CT * nf; idx += blockDim.x) {
      const int r = idx % CT, c = idx / CT;
      Fi[r * lds + c] = r < ri ? raw[c * CT + r] : 0.0;
      Fj[r * lds + c] = r < rj ? raw[(nf + c) * CT + r] : 0.0;
    }
  } else {
    load_feats(Fi, lds, F, ldf, i0, n, nf);
    load_feats(Fj, lds, F, ldf, j0, n, nf);
  }
  __syncthreads();
  const int r = threadIdx.x % CT;
  const int cb = threadIdx.x / CT;
  const int64_t i = i0 + r;
  const bool do_mirror = bi != bj;
  double kv[MT];
  double dv[MT][GPGP_TERM_NPARAM];
#pragma unroll 1
  for (int q = 0; q < CT / 4; ++q) {
    const int c = cb + 4 * q;
    const int64_t j = j0 + c;
    double v = 0.0;
    if (i < n && j < n) {
#pragma unroll
      for (int t = 0; t < MT; ++t)
        if (t < nterms)
          kv[t] = term_value_grad(dk.t[t], Fi + r * lds + dk.t[t].off, Fj + c * lds + dk.t[t].off, dv[t]);
      // the sum over groups of the products of their terms, in kernel_value's order
      double sum = 0.0, prod = 1.0;
      int g = dk.t[0].group;
#pragma unroll
      for (int t = 0; t < MT; ++t) {
        if (t >= nterms) break;
        if (dk.t[t].group != g) {
          sum += prod;
          prod = 1.0;
          g = dk.t[t].group;
        }
        prod *= kv[t];
      }
      sum += prod;
      v = (i == j) ? sum + jitter : sum;
      K[i + j * ldk] = v;
      if (i >= j) {
#pragma unroll
        for (int mi = 0; mi < GPGP_GRAD_MAXMAT; ++mi) {
          if (mi >= gm.nmat) break;
          const int ga = gm.grp[mi];
          double val = 1.0, dsel = 0.0;
#pragma unroll
          for (int t = 0; t < MT; ++t) {
            if (t >= nterms) break;
            if (dk.t[t].group != ga) continue;
            if (gm.kind[mi] == 1 && t == gm.a[mi]) {
#pragma unroll
              for (int p = 0; p < GPGP_TERM_NPARAM; ++p)
                if (p == gm.b[mi]) dsel = dv[t][p];
            } else {
              val *= kv[t];
            }
          }
          if (gm.kind[mi] == 1) val *= dsel;
          D[mi * dstride + i + j * ldd] = val;
        }
      }
    }
    if (do_mirror) Tt[c * (CT + 1) + r] = v;
  }
  if (do_mirror) {
    __syncthreads();
#pragma unroll 1
    for (int q = 0; q < CT / 4; ++q) {
      const int rr = threadIdx.x % CT;
      const int cc = threadIdx.x / CT + 4 * q;
      const int64_t jj = j0 + rr, ii = i0 + cc;
      if (jj < n && ii < n) K[jj + ii * ldk] = Tt[rr * (CT + 1) + cc];
    }
  }
}

void cov_matrix_grad(cudaStream_t s, const DevKernel &dk, const GradPlan &pl, const double *F, int64_t ldf,
                     int64_t n, double *K, int64_t ldk, double jitter, double *D, int64_t ldd, int64_t dstride,
                     int *err) {
  if (n == 0) return;
  const int lds = (dk.nfeat | 1);
  if (!(err && dk.nfeat <= 64 && bulk_ok(F, ldf, n))) err = nullptr;
  const size_t smem = (size_t)(2 * CT * lds + CT * (CT + 1)) * sizeof(double) +
                      (err ? (size_t)2 * dk.nfeat * CT * sizeof(double) + 16 : 0);
  static PerDevice attr;
  per_device(attr, [] {
    const int mx = 2 * CT * 65 * 8 + CT * (CT + 1) * 8 + 2 * 64 * CT * 8 + 16;
    GPGP_CUDA(cudaFuncSetAttribute(cov_tile_grad_kernel<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx));
    GPGP_CUDA(cudaFuncSetAttribute(cov_tile_grad_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx));
    GPGP_CUDA(cudaFuncSetAttribute(cov_tile_grad_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx));
    GPGP_CUDA(cudaFuncSetAttribute(cov_tile_grad_kernel<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx));
    return 1;
  });
  const int64_t T = (n + CT - 1) / CT;
  const unsigned nt = (unsigned)(T * (T + 1) / 2);
  switch (dk.nterms) {
    case 1:
      cov_tile_grad_kernel<1><<<nt, 256, smem, s>>>(dk, pl.m, F, ldf, n, K, ldk, jitter, D, ldd, dstride, err);
      break;
    case 2:
      cov_tile_grad_kernel<2><<<nt, 256, smem, s>>>(dk, pl.m, F, ldf, n, K, ldk, jitter, D, ldd, dstride, err);
      break;
    case 3:
      cov_tile_grad_kernel<3><<<nt, 256, smem, s>>>(dk, pl.m, F, ldf, n, K, ldk, jitter, D, ldd, dstride, err);
      break;
    default:
      cov_tile_grad_kernel<0><<<nt, 256, smem, s>>>(dk, pl.m, F, ldf, n, K, ldk, jitter, D, ldd, dstride, err);
  }
  GPGP_CHECK_LAUNCH();
}

// Contraction with the stored matrices. Per lower tile: W_ij = alpha_i alpha_j -
// s_i s_j Binv_ij (Binv given by its lower triangle, ldb), counted twice off the
// diagonal; part[tile (nmat + 1) + q] = sum W_ij D_q(i, j) for q < nmat and
// part[tile (nmat + 1) + nmat] = sum W_ij. Warp-shuffle sums in a fixed order,
// then the block's eight warps in order.
template <int NM>
__global__ void __launch_bounds__(256) grad_stored_kernel(int nmat, const double *__restrict__ Bi, int64_t ldb,
                                                          int64_t n, const double *__restrict__ alpha,
                                                          const double *__restrict__ sv, const double *__restrict__ D,
                                                          int64_t ldd, int64_t dstride, double *__restrict__ part) {
  constexpr int MM = NM > 0 ? NM : GPGP_GRAD_MAXMAT;
  const int nm = NM > 0 ? NM : nmat;
  __shared__ double red[8][MM + 1];
  int64_t bi, bj;
  tri_index(blockIdx.x, &bi, &bj);
  const int64_t i0 = bi * CT, j0 = bj * CT;
  const int r = threadIdx.x % CT;
  const int cb = threadIdx.x / CT;
  const int64_t i = i0 + r;
  double acc[MM + 1];
#pragma unroll
  for (int q = 0; q <= MM; ++q) acc[q] = 0.0;
  if (i < n) {
    const double ai = alpha[i], si = sv[i];
#pragma unroll 4
    for (int q = 0; q < CT / 4; ++q) {
      const int64_t j = j0 + cb + 4 * q;
      if (j > i) continue;
      const double w = (ai * alpha[j] - si * sv[j] * Bi[i + j * ldb]) * (i == j ? 1.0 : 2.0);
      acc[MM] += w;
#pragma unroll
      for (int mi = 0; mi < MM; ++mi)
        if (mi < nm) acc[mi] = fma(w, D[mi * dstride + i + j * ldd], acc[mi]);
    }
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q <= MM; ++q) {
    double v = acc[q];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    if (lane == 0) red[warp][q] = v;
  }
  __syncthreads();
  if (threadIdx.x <= nm) {
    const int q = threadIdx.x < nm ? threadIdx.x : MM;
    double t = red[0][q];
    for (int w = 1; w < 8; ++w) t += red[w][q];
    part[(int64_t)blockIdx.x * (nm + 1) + threadIdx.x] = t;
  }
}

// The same contraction in double-float arithmetic (mixed precision): per entry
// ~100 FP32 and integer operations where the FP64 kernel spends 7 FP64 ones (the
// FP64 pipe of this part retires 1/64 of the FP32 pipe's lane operations), so
// the kernel is bound by its reads. Each thread sums its 16 entries as pairs; the
// block's sums are formed in FP64 in the fixed order of grad_stored_kernel.
template <int NM>
__global__ void __launch_bounds__(256) grad_stored_df_kernel(int nmat, const double *__restrict__ Bi, int64_t ldb,
                                                             int64_t n, const double *__restrict__ alpha,
                                                             const double *__restrict__ sv,
                                                             const double *__restrict__ D, int64_t ldd,
                                                             int64_t dstride, double *__restrict__ part) {
  constexpr int MM = NM > 0 ? NM : GPGP_GRAD_MAXMAT;
  const int nm = NM > 0 ? NM : nmat;
  __shared__ double red[8][MM + 1];
  __shared__ f2 aj_s[CT], sj_s[CT];
  int64_t bi, bj;
  tri_index(blockIdx.x, &bi, &bj);
  const int64_t i0 = bi * CT, j0 = bj * CT;
  if (threadIdx.x < CT) {
    const int64_t j = j0 + threadIdx.x;
    aj_s[threadIdx.x] = j < n ? f2_of(alpha[j]) : f2{0.0f, 0.0f};
    sj_s[threadIdx.x] = j < n ? f2_of(sv[j]) : f2{0.0f, 0.0f};
  }
  __syncthreads();
  const int r = threadIdx.x % CT;
  const int cb = threadIdx.x / CT;
  const int64_t i = i0 + r;
  f2 acc[MM + 1];
#pragma unroll
  for (int q = 0; q <= MM; ++q) acc[q] = f2{0.0f, 0.0f};
  if (i < n) {
    const f2 ai = f2_of(alpha[i]), si = f2_of(sv[i]);
#pragma unroll 4
    for (int q = 0; q < CT / 4; ++q) {
      const int c = cb + 4 * q;
      const int64_t j = j0 + c;
      if (j > i) continue;
      const f2 t = f2_mul(f2_mul(si, sj_s[c]), f2_of(Bi[i + j * ldb]));
      f2 w = f2_add(f2_mul(ai, aj_s[c]), f2_neg(t));
      if (i != j) w = f2{2.0f * w.h, 2.0f * w.l};
      acc[MM] = f2_add(acc[MM], w);
#pragma unroll
      for (int mi = 0; mi < MM; ++mi)
        if (mi < nm) acc[mi] = f2_fma(w, f2_of(D[mi * dstride + i + j * ldd]), acc[mi]);
    }
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q <= MM; ++q) {
    double v = f2_to_double(acc[q]);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    if (lane == 0) red[warp][q] = v;
  }
  __syncthreads();
  if (threadIdx.x <= nm) {
    const int q = threadIdx.x < nm ? threadIdx.x : MM;
    double t = red[0][q];
    for (int w = 1; w < 8; ++w) t += red[w][q];
    part[(int64_t)blockIdx.x * (nm + 1) + threadIdx.x] = t;
  }
}

int64_t grad_stored_partials(int64_t n) {
  const int64_t T = (n + CT - 1) / CT;
  return T * (T + 1) / 2 * (GPGP_GRAD_MAXMAT + 1);
}

void grad_stored_contract(cudaStream_t s, const GradPlan &pl, int64_t n, const double *Bi, int64_t ldb,
                          const double *alpha, const double *sv, const double *D, int64_t ldd, int64_t dstride,
                          double *part, double *g, bool df) {
  const int64_t T = (n + CT - 1) / CT;
  const unsigned nt = (unsigned)(T * (T + 1) / 2);
  const int nm = pl.m.nmat;
  if (df) {
    switch (nm) {
      case 1:
        grad_stored_df_kernel<1><<<nt, 256, 0, s>>>(nm, Bi, ldb, n, alpha, sv, D, ldd, dstride, part);
        break;
      case 2:
        grad_stored_df_kernel<2><<<nt, 256, 0, s>>>(nm, Bi, ldb, n, alpha, sv, D, ldd, dstride, part);
        break;
      case 3:
        grad_stored_df_kernel<3><<<nt, 256, 0, s>>>(nm, Bi, ldb, n, alpha, sv, D, ldd, dstride, part);
        break;
      default:
        grad_stored_df_kernel<0><<<nt, 256, 0, s>>>(nm, Bi, ldb, n, alpha, sv, D, ldd, dstride, part);
    }
    GPGP_CHECK_LAUNCH();
    reduce_partials_kernel<<<1, 256, 0, s>>>(part, nt, nm + 1, g);
    GPGP_CHECK_LAUNCH();
    return;
  }
  switch (nm) {
    case 1:
      grad_stored_kernel<1><<<nt, 256, 0, s>>>(nm, Bi, ldb, n, alpha, sv, D, ldd, dstride, part);
      break;
    case 2:
      grad_stored_kernel<2><<<nt, 256, 0, s>>>(nm, Bi, ldb, n, alpha, sv, D, ldd, dstride, part);
      break;
    case 3:
      grad_stored_kernel<3><<<nt, 256, 0, s>>>(nm, Bi, ldb, n, alpha, sv, D, ldd, dstride, part);
      break;
    default:
      grad_stored_kernel<0><<<nt, 256, 0, s>>>(nm, Bi, ldb, n, alpha, sv, D, ldd, dstride, part);
  }
  GPGP_CHECK_LAUNCH();
  reduce_partials_kernel<<<1, 256, 0, s>>>(part, nt, nm + 1, g);
  GPGP_CHECK_LAUNCH();
}

void grad_stored_assemble(const GradPlan &pl, int nterms, const double *g, double *hg) {
  for (int idx = 0; idx < nterms * GPGP_TERM_NPARAM; ++idx) {
    const int q = pl.slot_mat[idx];
    hg[idx] = q == -2 ? 0.0 : pl.slot_scale[idx] * g[q >= 0 ? q : pl.m.nmat];
  }
}

// ---------------------------------------------------------------------------
// K (and its derivative matrices) in double-float arithmetic (mixed precision)
// ---------------------------------------------------------------------------
// The FP64 tile kernels above are bound by this part's FP64 pipe (~35 FP64
// operations per matern52 pair). Under mixed precision the covariance is instead
// evaluated in pair arithmetic (dfloat.cuh) on the FP32 pipe, which retires 64
// times the lane operations: the distance, its square root, the exponential
// and the polynomial factor, each to ~2^-44 relative, then converted to doubles
// without FP64 instructions. That is far below the ~2^-33 the sliced
// factorisation carries. Kernels made only of cf_const, cf_sexp, cf_matern32 and
// cf_matern52 terms (without periodic inputs) take this path.
bool cov_df_eligible(const DevKernel &dk) {
  for (int t = 0; t < dk.nterms; ++t) {
    const DevTerm &T = dk.t[t];
    if (T.periodic || (T.kind != GPGP_CF_CONST && T.kind != GPGP_CF_SEXP && T.kind != GPGP_CF_MATERN32 &&
                       T.kind != GPGP_CF_MATERN52))
      return false;
  }
  return true;
}

// One term's value and its derivatives with respect to log lscale (dv0) and log
// magn (dv1 = 2 k) as pairs; m2 and c1 are the term's constants as pairs.
template <bool GRAD>
__device__ __forceinline__ f2 term_value_df(int kind, f2 m2, f2 c1, const f2 *fi, const f2 *fj, int dt, f2 *dv0) {
  if (kind == GPGP_CF_CONST) return m2;
  // squared distance: each difference as a pair, its square as a pair, summed
  f2 r2 = f2{0.0f, 0.0f};
  for (int c = 0; c < dt; ++c) {
    const f2 a = fi[c], b = fj[c];
    const f2 dh = f2_two_sum(a.h, -b.h);
    const f2 df = f2_fast_two_sum(dh.h, __fadd_rn(dh.l, __fsub_rn(a.l, b.l)));
    r2 = f2_fma(df, df, r2);
  }
  if (kind == GPGP_CF_SEXP) {
    const f2 q = f2_mul(r2, c1);  // r^2 / lscale^2
    const f2 k = f2_mul(m2, f2_exp_neg(f2{-0.5f * q.h, -0.5f * q.l}));
    if (GRAD) *dv0 = f2_mul(k, q);
    return k;
  }
  const f2 a = f2_mul(c1, f2_sqrt(r2));
  const f2 me = f2_mul(m2, f2_exp_neg(f2_neg(a)));
  const f2 a2 = f2_mul(a, a);
  if (kind == GPGP_CF_MATERN32) {
    if (GRAD) *dv0 = f2_mul(me, a2);
    return f2_fma(me, a, me);  // m2 (1 + a) e^-a
  }
  const f2 a2_3 = f2_mul(a2, f2{0x1.555556p-2f, -0x1.555556p-27f});  // a^2 / 3
  if (GRAD) *dv0 = f2_mul(me, f2_fma(a2_3, a, a2_3));  // m2 a^2 (1 + a) / 3 e^-a
  return f2_mul(me, f2_add(f2_fast_two_sum(1.0f, 0.0f), f2_add(a, a2_3)));
}

// Lower 64 x 64 tiles of K = sum over groups of the products of their terms, with
// jitter on the diagonal, mirrored above it (cov_tile_kernel's layout); with GRAD,
// also the planned derivative matrices (entries i >= j); with Bout, also the lower
// triangle of B = I + s2 K (a constant scale, lik_gaussian: s2 = 1/sigma^2), so that
// the Cholesky starts from these tiles without a pass of its own over K.
// The tile's feature rows are staged in shared memory by the TMA unit: one bulk
// copy (cp.async.bulk) per feature column and tile, completing on an mbarrier,
// when every copy is 16-byte aligned and a multiple of 16 bytes long (even n and
// leading dimension); otherwise by plain loads. The wait is bounded: on timeout
// the kernel records it in *err (1), lets the copies land (bounded) and returns.
struct DfArgs {
  const double *F;
  int64_t ldf, n;
  double *K;
  int64_t ldk;
  double jitter;
  double *D;
  int64_t ldd, dstride;
  double *B;  // null: no B
  int64_t ldb;
  double s2;
  int bulk;   // 1: TMA staging allowed
  int *err;
};

template <int NT, bool GRAD>
__global__ void __launch_bounds__(256) cov_tile_df_kernel(DevKernel dk, GradMats gm, DfArgs g) {
  extern __shared__ __align__(16) double smd[];
  constexpr int MT = NT > 0 ? NT : GPGP_MAX_TERMS;
  const int nterms = NT > 0 ? NT : dk.nterms;
  const int nf = dk.nfeat;
  const int lds = (nf | 1);
  const int64_t n = g.n;
  int64_t bi, bj;
  tri_index(blockIdx.x, &bi, &bj);
  const int64_t i0 = bi * CT, j0 = bj * CT;
  const bool do_mirror = bi != bj;
  // shared memory: raw feature columns [2][nf][CT] doubles (TMA destination), the
  // mbarrier, the pair tiles, the mirror staging
  double *raw = smd;
  uint64_t *bar = reinterpret_cast<uint64_t *>(raw + 2 * nf * CT);
  f2 *Fi = reinterpret_cast<f2 *>(bar + 2);
  f2 *Fj = Fi + CT * lds;
  double *Tt = reinterpret_cast<double *>(Fj + CT * lds);  // CT x (CT+1) staging for the mirrored write
  const int64_t ri = n - i0 < CT ? n - i0 : CT, rj = n - j0 < CT ? n - j0 : CT;
  if (g.bulk) {
    // a diagonal tile needs its rows once
    if (!stage_features_bulk<CT>(raw, bar, g.F, g.ldf, i0, ri, g.F, g.ldf, j0, rj, do_mirror, nf, g.err)) return;
    for (int idx = threadIdx.x; idx < CT * nf; idx += blockDim.x) {
      const int r = idx % CT, c = idx / CT;
      Fi[r * lds + c] = r < ri ? f2_of(raw[c * CT + r]) : f2{0.0f, 0.0f};
      Fj[r * lds + c] = r < rj ? f2_of(raw[((do_mirror ? nf : 0) + c) * CT + r]) : f2{0.0f, 0.0f};
    }
  } else {
    for (int idx = threadIdx.x; idx < CT * nf; idx += blockDim.x) {
      const int r = idx % CT, c = idx / CT;
      Fi[r * lds + c] = r < ri ? f2_of(g.F[i0 + r + c * g.ldf]) : f2{0.0f, 0.0f};
      Fj[r * lds + c] = r < rj ? f2_of(g.F[j0 + r + c * g.ldf]) : f2{0.0f, 0.0f};
    }
  }
  f2 m2[MT], c1[MT];
#pragma unroll
  for (int t = 0; t < MT; ++t) {
    if (t < nterms) {
      m2[t] = f2_of(dk.t[t].m2);
      c1[t] = f2_of(dk.t[t].c1);
    }
  }
  const f2 s2 = f2_of(g.s2);
  __syncthreads();
  const int r = threadIdx.x % CT;
  const int cb = threadIdx.x / CT;
  const int64_t i = i0 + r;
  f2 kv[MT], dv0[MT];
#pragma unroll 1
  for (int q = 0; q < CT / 4; ++q) {
    const int c = cb + 4 * q;
    const int64_t j = j0 + c;
    double v = 0.0;
    if (i < n && j < n) {
#pragma unroll
      for (int t = 0; t < MT; ++t)
        if (t < nterms)
          kv[t] = term_value_df<GRAD>(dk.t[t].kind, m2[t], c1[t], Fi + r * lds + dk.t[t].off,
                                      Fj + c * lds + dk.t[t].off, dk.t[t].dt, &dv0[t]);
      f2 sum = f2{0.0f, 0.0f}, prod = f2{1.0f, 0.0f};
      int grp = dk.t[0].group;
#pragma unroll
      for (int t = 0; t < MT; ++t) {
        if (t >= nterms) break;
        if (dk.t[t].group != grp) {
          sum = f2_add(sum, prod);
          prod = f2{1.0f, 0.0f};
          grp = dk.t[t].group;
        }
        prod = t == 0 || dk.t[t - 1].group != dk.t[t].group ? kv[t] : f2_mul(prod, kv[t]);
      }
      sum = f2_add(sum, prod);
      v = f2_to_double(sum);  // the jitter is added below, outside the pair loop
      g.K[i + j * g.ldk] = v;
      if (g.B && i > j) g.B[i + j * g.ldb] = f2_to_double(f2_mul(sum, s2));
      if (GRAD && i >= j) {
#pragma unroll
        for (int mi = 0; mi < GPGP_GRAD_MAXMAT; ++mi) {
          if (mi >= gm.nmat) break;
          const int ga = gm.grp[mi];
          f2 val = f2{1.0f, 0.0f};
          bool first = true;
#pragma unroll
          for (int t = 0; t < MT; ++t) {
            if (t >= nterms) break;
            if (dk.t[t].group != ga) continue;
            // kind 1: the slot's derivative in place of its term (lscale: dv0;
            // magnitude slots are kind 0, the group value)
            const f2 f = (gm.kind[mi] == 1 && t == gm.a[mi]) ? dv0[t] : kv[t];
            val = first ? f : f2_mul(val, f);
            first = false;
          }
          g.D[mi * g.dstride + i + j * g.ldd] = f2_to_double(val);
        }
      }
    }
    if (do_mirror) Tt[c * (CT + 1) + r] = v;
  }
  if (do_mirror) {
    __syncthreads();
#pragma unroll 1
    for (int q = 0; q < CT / 4; ++q) {
      const int rr = threadIdx.x % CT;
      const int cc = threadIdx.x / CT + 4 * q;
      const int64_t jj = j0 + rr, ii = i0 + cc;
      if (jj < n && ii < n) g.K[jj + ii * g.ldk] = Tt[rr * (CT + 1) + cc];
    }
  } else {
    // diagonal tile: the jitter, once per diagonal entry (written above by the
    // thread with c == r, visible to the block after the barrier), and B's diagonal
    __syncthreads();
    if (threadIdx.x < CT && i0 + threadIdx.x < n) {
      const int64_t d = i0 + threadIdx.x;
      const double kd = g.K[d * (g.ldk + 1)] + g.jitter;
      g.K[d * (g.ldk + 1)] = kd;
      if (g.B) g.B[d * (g.ldb + 1)] = 1.0 + g.s2 * kd;
    }
  }
}

template <bool GRAD>
static void launch_cov_df(cudaStream_t s, const DevKernel &dk, const GradMats &gm, const DfArgs &a) {
  const int lds = (dk.nfeat | 1);
  const size_t smem = (size_t)2 * dk.nfeat * CT * sizeof(double) + 16 + (size_t)(2 * CT * lds) * sizeof(f2) +
                      (size_t)CT * (CT + 1) * sizeof(double);
  static PerDevice attr;
  per_device(attr, [] {
    const int mx = 2 * 64 * CT * 8 + 16 + 2 * CT * 65 * 8 + CT * (CT + 1) * 8;
    GPGP_CUDA(cudaFuncSetAttribute(cov_tile_df_kernel<0, GRAD>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx));
    GPGP_CUDA(cudaFuncSetAttribute(cov_tile_df_kernel<1, GRAD>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx));
    GPGP_CUDA(cudaFuncSetAttribute(cov_tile_df_kernel<2, GRAD>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx));
    GPGP_CUDA(cudaFuncSetAttribute(cov_tile_df_kernel<3, GRAD>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx));
    return 1;
  });
  const int64_t T = (a.n + CT - 1) / CT;
  const unsigned nt = (unsigned)(T * (T + 1) / 2);
  switch (dk.nterms) {
    case 1:
      cov_tile_df_kernel<1, GRAD><<<nt, 256, smem, s>>>(dk, gm, a);
      break;
    case 2:
      cov_tile_df_kernel<2, GRAD><<<nt, 256, smem, s>>>(dk, gm, a);
      break;
    case 3:
      cov_tile_df_kernel<3, GRAD><<<nt, 256, smem, s>>>(dk, gm, a);
      break;
    default:
      cov_tile_df_kernel<0, GRAD><<<nt, 256, smem, s>>>(dk, gm, a);
  }
  GPGP_CHECK_LAUNCH();
}

void cov_matrix_df(cudaStream_t s, const DevKernel &dk, const GradPlan *pl, const double *F, int64_t ldf, int64_t n,
                   double *K, int64_t ldk, double jitter, double *D, int64_t ldd, int64_t dstride, int *err,
                   double *B, int64_t ldb, double s2) {
  if (n == 0) return;
  DfArgs a;
  a.F = F;
  a.ldf = ldf;
  a.n = n;
  a.K = K;
  a.ldk = ldk;
  a.jitter = jitter;
  a.D = D;
  a.ldd = ldd;
  a.dstride = dstride;
  a.B = B;
  a.ldb = ldb;
  a.s2 = s2;
  // every bulk copy starts on a 16-byte boundary and moves a multiple of 16 bytes
  a.bulk = (err && dk.nfeat <= 64 && bulk_ok(F, ldf, n)) ? 1 : 0;
  a.err = err;
  if (pl) {
    launch_cov_df<true>(s, dk, pl->m, a);
  } else {
    GradMats none;
    std::memset(&none, 0, sizeof(none));
    launch_cov_df<false>(s, dk, none, a);
  }
}

// K(x1_i, x2_j) as a pair: the sum over the groups selected by gmask of the
// products of their terms (kernel_value's order).
template <int NT>
__device__ __forceinline__ f2 kernel_value_df(const DevKernel &dk, uint32_t gmask, const f2 *m2, const f2 *c1,
                                              const f2 *fi, const f2 *fj) {
  constexpr int MT = NT > 0 ? NT : GPGP_MAX_TERMS;
  const int nterms = NT > 0 ? NT : dk.nterms;
  f2 sum = f2{0.0f, 0.0f}, prod = f2{1.0f, 0.0f};
  int g = dk.t[0].group;
  bool first = true;
#pragma unroll
  for (int t = 0; t < MT; ++t) {
    if (t >= nterms) break;
    if (dk.t[t].group != g) {
      if (gmask & (1u << g)) sum = f2_add(sum, prod);
      prod = f2{1.0f, 0.0f};
      g = dk.t[t].group;
      first = true;
    }
    if (gmask & (1u << g)) {
      const f2 kv = term_value_df<false>(dk.t[t].kind, m2[t], c1[t], fi + dk.t[t].off, fj + dk.t[t].off,
                                         dk.t[t].dt, nullptr);
      prod = first ? kv : f2_mul(prod, kv);
      first = false;
    }
  }
  if (gmask & (1u << g)) sum = f2_add(sum, prod);
  return sum;
}

template <int MT>
__device__ __forceinline__ void load_consts_df(const DevKernel &dk, int nterms, f2 *m2, f2 *c1) {
#pragma unroll
  for (int t = 0; t < MT; ++t) {
    if (t < nterms) {
      m2[t] = f2_of(dk.t[t].m2);
      c1[t] = f2_of(dk.t[t].c1);
    }
  }
}

// Cross covariance out_ij = s_i K(x1_i, x2_j) (s null: 1), 64 x 64 tiles (grid T1 x T2).
template <int NT>
__global__ void __launch_bounds__(256) cov_cross_df_kernel(DevKernel dk, uint32_t gmask, const double *__restrict__ F1,
                                                           int64_t ld1, int64_t n1, const double *__restrict__ F2,
                                                           int64_t ld2, int64_t n2, double *__restrict__ out,
                                                           int64_t ldo, const double *__restrict__ scale) {
  extern __shared__ double smd[];
  constexpr int MT = NT > 0 ? NT : GPGP_MAX_TERMS;
  const int nterms = NT > 0 ? NT : dk.nterms;
  const int nf = dk.nfeat;
  const int lds = (nf | 1);
  f2 *Fi = reinterpret_cast<f2 *>(smd);
  f2 *Fj = Fi + CT * lds;
  const int64_t i0 = (int64_t)blockIdx.x * CT, j0 = (int64_t)blockIdx.y * CT;
  for (int idx = threadIdx.x; idx < CT * nf; idx += blockDim.x) {
    const int r = idx % CT, c = idx / CT;
    Fi[r * lds + c] = i0 + r < n1 ? f2_of(F1[i0 + r + c * ld1]) : f2{0.0f, 0.0f};
    Fj[r * lds + c] = j0 + r < n2 ? f2_of(F2[j0 + r + c * ld2]) : f2{0.0f, 0.0f};
  }
  f2 m2[MT], c1[MT];
  load_consts_df<MT>(dk, nterms, m2, c1);
  __syncthreads();
  const int r = threadIdx.x % CT;
  const int cb = threadIdx.x / CT;
  const int64_t i = i0 + r;
  if (i >= n1) return;
  const f2 si = scale ? f2_of(scale[i]) : f2{1.0f, 0.0f};
#pragma unroll 1
  for (int q = 0; q < CT / 4; ++q) {
    const int c = cb + 4 * q;
    const int64_t j = j0 + c;
    if (j >= n2) continue;
    const f2 v = kernel_value_df<NT>(dk, gmask, m2, c1, Fi + r * lds, Fj + c * lds);
    out[i + j * ldo] = f2_to_double(scale ? f2_mul(si, v) : v);
  }
}

void cov_cross_df(cudaStream_t s, const DevKernel &dk, uint32_t gmask, const double *F1, int64_t ld1, int64_t n1,
                  const double *F2, int64_t ld2, int64_t n2, double *out, int64_t ldo, const double *scale) {
  if (n1 == 0 || n2 == 0) return;
  const int lds = (dk.nfeat | 1);
  const size_t smem = (size_t)(2 * CT * lds) * sizeof(f2);
  static PerDevice attr;
  per_device(attr, [] {
    const int mx = 2 * CT * 65 * 8;
    GPGP_CUDA(cudaFuncSetAttribute(cov_cross_df_kernel<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx));
    GPGP_CUDA(cudaFuncSetAttribute(cov_cross_df_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx));
    GPGP_CUDA(cudaFuncSetAttribute(cov_cross_df_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx));
    GPGP_CUDA(cudaFuncSetAttribute(cov_cross_df_kernel<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx));
    return 1;
  });
  const dim3 grid((unsigned)((n1 + CT - 1) / CT), (unsigned)((n2 + CT - 1) / CT));
  switch (dk.nterms) {
    case 1:
      cov_cross_df_kernel<1><<<grid, 256, smem, s>>>(dk, gmask, F1, ld1, n1, F2, ld2, n2, out, ldo, scale);
      break;
    case 2:
      cov_cross_df_kernel<2><<<grid, 256, smem, s>>>(dk, gmask, F1, ld1, n1, F2, ld2, n2, out, ldo, scale);
      break;
    case 3:
      cov_cross_df_kernel<3><<<grid, 256, smem, s>>>(dk, gmask, F1, ld1, n1, F2, ld2, n2, out, ldo, scale);
      break;
    default:
      cov_cross_df_kernel<0><<<grid, 256, smem, s>>>(dk, gmask, F1, ld1, n1, F2, ld2, n2, out, ldo, scale);
  }
  GPGP_CHECK_LAUNCH();
}

// out[i] = sum_j K(x1_i, x2_j) v_j with the products accumulated as pairs: block
// (x, y) takes rows [x CT, (x+1) CT) and the y-th range of x2 tiles; with several
// ranges the partial sums go to out + y n1 (as cov_matvec_kernel).
template <int NT>
__global__ void __launch_bounds__(256) cov_matvec_df_kernel(DevKernel dk, uint32_t gmask, const double *__restrict__ F1,
                                                            int64_t ld1, int64_t n1, const double *__restrict__ F2,
                                                            int64_t ld2, int64_t n2, const double *__restrict__ v,
                                                            double *__restrict__ out, int64_t tiles_per_range) {
  extern __shared__ double smd[];
  constexpr int MT = NT > 0 ? NT : GPGP_MAX_TERMS;
  const int nterms = NT > 0 ? NT : dk.nterms;
  const int nf = dk.nfeat;
  const int lds = (nf | 1);
  f2 *Fi = reinterpret_cast<f2 *>(smd);
  f2 *Fj = Fi + CT * lds;
  f2 *vj = Fj + CT * lds;
  f2 *red = vj + CT;  // 4 x CT partial pairs
  const int64_t i0 = (int64_t)blockIdx.x * CT;
  out += (int64_t)blockIdx.y * n1;
  for (int idx = threadIdx.x; idx < CT * nf; idx += blockDim.x) {
    const int r = idx % CT, c = idx / CT;
    Fi[r * lds + c] = i0 + r < n1 ? f2_of(F1[i0 + r + c * ld1]) : f2{0.0f, 0.0f};
  }
  f2 m2[MT], c1[MT];
  load_consts_df<MT>(dk, nterms, m2, c1);
  const int r = threadIdx.x % CT;
  const int cb = threadIdx.x / CT;
  f2 acc = f2{0.0f, 0.0f};
  const int64_t jbeg = (int64_t)blockIdx.y * tiles_per_range * CT;
  const int64_t jlim = jbeg + tiles_per_range * CT;
  const int64_t jend = jlim < n2 ? jlim : n2;
  for (int64_t j0 = jbeg; j0 < jend; j0 += CT) {
    __syncthreads();
    for (int idx = threadIdx.x; idx < CT * nf; idx += blockDim.x) {
      const int rr = idx % CT, c = idx / CT;
      Fj[rr * lds + c] = j0 + rr < n2 ? f2_of(F2[j0 + rr + c * ld2]) : f2{0.0f, 0.0f};
    }
    if (threadIdx.x < CT) vj[threadIdx.x] = (j0 + threadIdx.x < n2) ? f2_of(v[j0 + threadIdx.x]) : f2{0.0f, 0.0f};
    __syncthreads();
    if (i0 + r < n1) {
#pragma unroll 1
      for (int q = 0; q < CT / 4; ++q) {
        const int c = cb * (CT / 4) + q;
        if (j0 + c < n2) acc = f2_fma(kernel_value_df<NT>(dk, gmask, m2, c1, Fi + r * lds, Fj + c * lds), vj[c], acc);
      }
    }
  }
  red[cb * CT + r] = acc;
  __syncthreads();
  if (threadIdx.x < CT && i0 + threadIdx.x < n1) {
    f2 t = red[threadIdx.x];
    for (int k = 1; k < 4; ++k) t = f2_add(t, red[k * CT + threadIdx.x]);
    out[i0 + threadIdx.x] = f2_to_double(t);
  }
}

void cov_matvec_df(cudaStream_t s, const DevKernel &dk, uint32_t gmask, const double *F1, int64_t ld1, int64_t n1,
                   const double *F2, int64_t ld2, int64_t n2, const double *v, double *out) {
  if (n1 == 0) return;
  const int lds = (dk.nfeat | 1);
  const size_t smem = (size_t)(2 * CT * lds + CT + 4 * CT) * sizeof(f2);
  static PerDevice attr;
  per_device(attr, [] {
    const int mx = (2 * CT * 65 + 5 * CT) * 8;
    GPGP_CUDA(cudaFuncSetAttribute(cov_matvec_df_kernel<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx));
    GPGP_CUDA(cudaFuncSetAttribute(cov_matvec_df_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx));
    GPGP_CUDA(cudaFuncSetAttribute(cov_matvec_df_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx));
    GPGP_CUDA(cudaFuncSetAttribute(cov_matvec_df_kernel<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx));
    return 1;
  });
  const int64_t T1 = (n1 + CT - 1) / CT, T2 = std::max<int64_t>(1, (n2 + CT - 1) / CT);
  // four blocks per SM: the pair arithmetic needs the warps to hide its latency
  // (two per SM left the FP32 pipe at 56%)
  const int64_t want = std::max<int64_t>(1, (4 * device_sms() + T1 - 1) / T1);
  const int64_t tpr = (T2 + std::min(want, T2) - 1) / std::min(want, T2);
  const int64_t nrange = (T2 + tpr - 1) / tpr;
  double *dst = out, *part = nullptr;
  if (nrange > 1) {
    GPGP_CUDA(cudaMallocAsync((void **)&part, (size_t)nrange * n1 * sizeof(double), s));
    dst = part;
  }
  const dim3 grid((unsigned)T1, (unsigned)nrange);
  switch (dk.nterms) {
    case 1:
      cov_matvec_df_kernel<1><<<grid, 256, smem, s>>>(dk, gmask, F1, ld1, n1, F2, ld2, n2, v, dst, tpr);
      break;
    case 2:
      cov_matvec_df_kernel<2><<<grid, 256, smem, s>>>(dk, gmask, F1, ld1, n1, F2, ld2, n2, v, dst, tpr);
      break;
    case 3:
      cov_matvec_df_kernel<3><<<grid, 256, smem, s>>>(dk, gmask, F1, ld1, n1, F2, ld2, n2, v, dst, tpr);
      break;
    default:
      cov_matvec_df_kernel<0><<<grid, 256, smem, s>>>(dk, gmask, F1, ld1, n1, F2, ld2, n2, v, dst, tpr);
  }
  GPGP_CHECK_LAUNCH();
  if (nrange > 1) {
    sum_ranges_kernel<<<(unsigned)((n1 + 255) / 256), 256, 0, s>>>(part, nrange, n1, out);
    GPGP_CHECK_LAUNCH();
    GPGP_CUDA(cudaFreeAsync(part, s));
  }
}

}  // namespace gpgp
