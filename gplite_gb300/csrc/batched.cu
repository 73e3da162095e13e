// Batched small GPs: thousands of independent Gaussian-likelihood, full-method
// fits of uneven size, each followed by the reference's LOO (gp_loo with
// approx_laplace, R/gp_loo.R:73-129) and a prediction (gp_pred_post.method_full,
// R/gp_pred.R:202-232), run as one CUDA graph.
//
// Problems are grouped into buckets by n rounded up to 64 and padded: the padded
// part of B = I + K / sigma^2 is the identity, so it adds nothing to the factor,
// the solves or the log-determinant, and every problem of a bucket can run the
// blocked algorithms of dense.cu / mixed.cu in lockstep (problem index on a grid
// axis). Each bucket's contractions run either on the FP64 pipe or through the
// BF16-sliced tcgen05 GEMM; a small autotuner times both on the first run of a
// mixed-precision plan and keeps the faster per bucket. The whole sequence is then
// captured once into a CUDA graph and replayed.
#include <math.h>

#include <algorithm>
#include <cstring>
#include <map>
#include <vector>

#include "common.cuh"
#include "dfloat.cuh"
#include "fp64math.cuh"
#include "model.cuh"

namespace gpgp {

// potrf_diag_kernel lives in dense.cu
__global__ void potrf_diag_kernel(double *__restrict__ A, int kb, int64_t lda,
                                  double *__restrict__ Winv, double *__restrict__ logdet_part,
                                  int *__restrict__ status, int64_t k0, int64_t sA, int64_t sW,
                                  int64_t sL);

namespace {

constexpr int PRM = 8;  // doubles per problem: n, m, d, kind, lscale, magn, sigma, -
constexpr int BT = 64;  // tile edge

struct Bucket {
  int64_t nb = 0, mb = 0, dm = 0, count = 0;
  std::vector<int> probs;
  DBuf prm, X, Y, Xt, Bm, Bc, Winv, ldp, W, R, T, tmp, alpha, fhat, lml, mean, var, loos, binv;
  IBuf status;
  // sliced operands of the tensor-core variant
  void *sa = nullptr, *sb = nullptr;
  OzSplit SA, SB;
  int variant = 0;  // 0: FP64 pipe; sliced tensor cores with 1: 64-wide, 2: 256-wide outer panels
  double best_ms = 0.0;  // the autotuner's time of the chosen variant
  ~Bucket() {
    if (sa) cudaFreeAsync(sa, X.s);
    if (sb) cudaFreeAsync(sb, X.s);
  }
};

__device__ __forceinline__ double bat_kernel(int kind, double lscale, double m2, const double *xi,
                                             int si, const double *xj, int sj, int d) {
  double r2 = 0.0;
  for (int k = 0; k < d; ++k) {
    const double df = xi[k * si] - xj[k * sj];
    r2 += df * df;
  }
  if (kind == GPGP_CF_SEXP) return m2 * exp_fast(-0.5 * r2 * (1.0 / (lscale * lscale)));
  const double c = (kind == GPGP_CF_MATERN32 ? sqrt(3.0) : sqrt(5.0)) / lscale;
  const double a = c * sqrt_fast(r2);
  if (kind == GPGP_CF_MATERN32) return m2 * (1.0 + a) * exp_fast(-a);
  return m2 * (1.0 + a + a * a * (1.0 / 3.0)) * exp_fast(-a);
}

// The same in double-float arithmetic (mixed-precision plans): c1 is 1/lscale^2
// (sexp) or sqrt(3 | 5)/lscale (Matern) as a pair; x as pairs.
__device__ __forceinline__ f2 bat_kernel_df(int kind, f2 c1, f2 m2, const f2 *xi, const f2 *xj, int d) {
  f2 r2 = f2{0.0f, 0.0f};
  for (int k = 0; k < d; ++k) {
    const f2 dh = f2_two_sum(xi[k].h, -xj[k].h);
    const f2 df = f2_fast_two_sum(dh.h, __fadd_rn(dh.l, __fsub_rn(xi[k].l, xj[k].l)));
    r2 = f2_fma(df, df, r2);
  }
  if (kind == GPGP_CF_SEXP) {
    const f2 q = f2_mul(r2, c1);
    return f2_mul(m2, f2_exp_neg(f2{-0.5f * q.h, -0.5f * q.l}));
  }
  const f2 a = f2_mul(c1, f2_sqrt(r2));
  const f2 me = f2_mul(m2, f2_exp_neg(f2_neg(a)));
  if (kind == GPGP_CF_MATERN32) return f2_fma(me, a, me);
  const f2 a2_3 = f2_mul(f2_mul(a, a), f2{0x1.555556p-2f, -0x1.555556p-27f});
  return f2_mul(me, f2_add(f2{1.0f, 0.0f}, f2_add(a, a2_3)));
}

__device__ __forceinline__ double bat_c1(int kind, double ls) {
  return kind == GPGP_CF_SEXP ? 1.0 / (ls * ls) : (kind == GPGP_CF_MATERN32 ? sqrt(3.0) : sqrt(5.0)) / ls;
}

// B = I + s (K + jitter I) s on the lower triangle; identity on the padding.
// With Bc given, the full symmetric B is also written there (the refinement's
// residuals read it), the transposed tile through shared memory.
// DF: K evaluated in double-float arithmetic (mixed-precision plans).
template <bool DF>
__global__ void __launch_bounds__(256) bat_cov_B_kernel(int64_t nb, int64_t dm, const double *__restrict__ X,
                                                        const double *__restrict__ prm, double jitter,
                                                        double *__restrict__ B, double *__restrict__ Bc) {
  __shared__ double xi[BT][9], xj[BT][9];
  __shared__ f2 fxi[DF ? BT : 1][9], fxj[DF ? BT : 1][9];
  __shared__ double tile[BT][BT + 1];
  const int64_t z = blockIdx.y;
  const double *p = prm + z * PRM;
  const int n = (int)p[0], d = (int)p[2], kind = (int)p[3];
  const double ls = p[4], m2 = p[5] * p[5], s = sqrt(1.0 / (p[6] * p[6]));
  int64_t bi = (int64_t)((sqrt(8.0 * blockIdx.x + 1.0) - 1.0) * 0.5), bj;
  while (bi * (bi + 1) / 2 > (int64_t)blockIdx.x) --bi;
  while ((bi + 1) * (bi + 2) / 2 <= (int64_t)blockIdx.x) ++bi;
  bj = blockIdx.x - bi * (bi + 1) / 2;
  const int64_t i0 = bi * BT, j0 = bj * BT;
  const double *Xz = X + z * nb * dm;
  for (int idx = threadIdx.x; idx < BT * 8; idx += 256) {
    const int r = idx % BT, k = idx / BT;
    xi[r][k] = (k < d && i0 + r < n) ? Xz[i0 + r + k * nb] : 0.0;
    xj[r][k] = (k < d && j0 + r < n) ? Xz[j0 + r + k * nb] : 0.0;
    if (DF) {
      fxi[r][k] = f2_of(xi[r][k]);
      fxj[r][k] = f2_of(xj[r][k]);
    }
  }
  __syncthreads();
  double *Bz = B + z * nb * nb;
  const int r = threadIdx.x % BT, cb = threadIdx.x / BT;
  const int64_t i = i0 + r;
  f2 dc1 = f2{0.0f, 0.0f}, dm2 = f2{0.0f, 0.0f}, ds2 = f2{0.0f, 0.0f};
  if (DF) {
    dc1 = f2_of(bat_c1(kind, ls));
    dm2 = f2_of(m2);
    ds2 = f2_of(s * s);
  }
  for (int q = 0; q < BT / 4; ++q) {
    const int c = cb + 4 * q;
    const int64_t j = j0 + c;
    double v;
    if (i < n && j < n) {
      if (DF) {
        // s^2 (K + jitter I) as a pair; the identity added in FP64
        f2 k = bat_kernel_df(kind, dc1, dm2, &fxi[r][0], &fxj[c][0], d);
        if (i == j) k = f2_add(k, f2_of(jitter));
        v = f2_to_double(f2_mul(k, ds2));
      } else {
        double k = bat_kernel(kind, ls, m2, &xi[r][0], 1, &xj[c][0], 1, d);
        if (i == j) k += jitter;
        v = s * (k * s);
      }
      if (i == j) v += 1.0;
    } else {
      v = (i == j) ? 1.0 : 0.0;
    }
    tile[r][c] = v;
    if (j <= i) Bz[i + j * nb] = v;
  }
  if (!Bc) return;
  __syncthreads();
  double *Cz = Bc + z * nb * nb;
  for (int q = 0; q < BT / 4; ++q) {
    const int c = cb + 4 * q;
    Cz[(i0 + r) + (j0 + c) * nb] = tile[r][c];
    if (bi != bj) Cz[(j0 + r) + (i0 + c) * nb] = tile[c][r];
  }
}

// R = s K(x, xt) (nb x mb per problem, zero on the padding); DF as above
template <bool DF>
__global__ void __launch_bounds__(256) bat_cross_kernel(int64_t nb, int64_t mb, int64_t dm,
                                                        const double *__restrict__ X,
                                                        const double *__restrict__ Xt,
                                                        const double *__restrict__ prm,
                                                        double *__restrict__ R) {
  __shared__ double xi[BT][9], xj[BT][9];
  __shared__ f2 fxi[DF ? BT : 1][9], fxj[DF ? BT : 1][9];
  const int64_t z = blockIdx.z;
  const double *p = prm + z * PRM;
  const int n = (int)p[0], m = (int)p[1], d = (int)p[2], kind = (int)p[3];
  const double ls = p[4], m2 = p[5] * p[5], s = sqrt(1.0 / (p[6] * p[6]));
  const int64_t i0 = (int64_t)blockIdx.x * BT, j0 = (int64_t)blockIdx.y * BT;
  const double *Xz = X + z * nb * dm, *Tz = Xt + z * mb * dm;
  for (int idx = threadIdx.x; idx < BT * 8; idx += 256) {
    const int r = idx % BT, k = idx / BT;
    xi[r][k] = (k < d && i0 + r < n) ? Xz[i0 + r + k * nb] : 0.0;
    xj[r][k] = (k < d && j0 + r < m) ? Tz[j0 + r + k * mb] : 0.0;
    if (DF) {
      fxi[r][k] = f2_of(xi[r][k]);
      fxj[r][k] = f2_of(xj[r][k]);
    }
  }
  __syncthreads();
  double *Rz = R + z * nb * mb;
  const int r = threadIdx.x % BT, cb = threadIdx.x / BT;
  const int64_t i = i0 + r;
  if (i >= nb) return;
  f2 dc1 = f2{0.0f, 0.0f}, dm2 = f2{0.0f, 0.0f}, ds = f2{0.0f, 0.0f};
  if (DF) {
    dc1 = f2_of(bat_c1(kind, ls));
    dm2 = f2_of(m2);
    ds = f2_of(s);
  }
  for (int q = 0; q < BT / 4; ++q) {
    const int64_t j = j0 + cb + 4 * q;
    if (j >= mb) continue;
    double v = 0.0;
    if (i < n && j < m) {
      if (DF)
        v = f2_to_double(f2_mul(ds, bat_kernel_df(kind, dc1, dm2, &fxi[r][0], &fxj[cb + 4 * q][0], d)));
      else
        v = s * bat_kernel(kind, ls, m2, &xi[r][0], 1, &xj[cb + 4 * q][0], 1, d);
    }
    Rz[i + j * nb] = v;
  }
}

// b := L^-T L^-1 b for one problem (the CTA's 256 threads; x is scratch of nb)
__device__ void bat_tri_solve(int64_t nb, const double *__restrict__ L, const double *__restrict__ Wz,
                              double *b, double *x, double *bk, double *xk) {
  const int tid = threadIdx.x;
  const int64_t nblk = nb / NB;
  for (int64_t k = 0; k < nblk; ++k) {  // forward: x = L^-1 b
    const int64_t k0 = k * NB;
    if (tid < NB) bk[tid] = b[k0 + tid];
    __syncthreads();
    if (tid < NB) {
      double acc = 0.0;
      for (int c = 0; c <= tid; ++c) acc = fma(Wz[k0 * NB + tid + c * NB], bk[c], acc);
      xk[tid] = acc;
      x[k0 + tid] = acc;
    }
    __syncthreads();
    for (int64_t r = k0 + NB + tid; r < nb; r += 256) {
      double acc = 0.0;
      for (int c = 0; c < NB; ++c) acc = fma(L[r + (k0 + c) * nb], xk[c], acc);
      b[r] -= acc;
    }
    __syncthreads();
  }
  for (int64_t k = nblk - 1; k >= 0; --k) {  // backward: b = L^-T x
    const int64_t k0 = k * NB;
    if (tid < NB) bk[tid] = x[k0 + tid];
    __syncthreads();
    if (tid < NB) {
      double acc = 0.0;
      for (int r = tid; r < NB; ++r) acc = fma(Wz[k0 * NB + r + tid * NB], bk[r], acc);
      xk[tid] = acc;
      b[k0 + tid] = acc;
    }
    __syncthreads();
    for (int64_t c = tid; c < k0; c += 256) {
      double acc = 0.0;
      for (int r = 0; r < NB; ++r) acc = fma(L[(k0 + r) + c * nb], xk[r], acc);
      x[c] -= acc;
    }
    __syncthreads();
  }
}

// alpha = s B^-1 (s y), fhat = y - sigma^2 alpha (= K alpha, C alpha = y); one CTA
// per problem. With Bc (the full FP64 B) the solve is refined iters times:
// u += B^-1 (s y - B u), the residual in FP64 and the correction through the
// factor, so that alpha reaches FP64 accuracy from a mixed-precision factor.
__global__ void __launch_bounds__(256) bat_solve_kernel(int64_t nb, const double *__restrict__ Lb,
                                                        const double *__restrict__ Winv,
                                                        const double *__restrict__ Bc, int iters,
                                                        const double *__restrict__ Y,
                                                        const double *__restrict__ prm,
                                                        const int *__restrict__ status, double *t1,
                                                        double *t2, double *t3, double *__restrict__ alpha,
                                                        double *__restrict__ fhat) {
  __shared__ double bk[NB], xk[NB];
  const int64_t z = blockIdx.x;
  if (status[z] != 0) return;
  const double *p = prm + z * PRM;
  const int n = (int)p[0];
  const double sig2 = p[6] * p[6], s = sqrt(1.0 / sig2);
  const double *L = Lb + z * nb * nb;
  const double *Wz = Winv + z * nb * NB;
  double *u = t1 + z * nb, *x = t2 + z * nb, *rr = t3 + z * nb;
  const int tid = threadIdx.x;
  for (int64_t i = tid; i < nb; i += 256) u[i] = i < n ? s * Y[z * nb + i] : 0.0;
  __syncthreads();
  bat_tri_solve(nb, L, Wz, u, x, bk, xk);
  if (Bc) {
    const double *Bz = Bc + z * nb * nb;
    for (int it = 0; it < iters; ++it) {
      for (int64_t i = tid; i < nb; i += 256) {
        double acc = i < n ? s * Y[z * nb + i] : 0.0;
        for (int64_t j = 0; j < nb; ++j) acc = fma(-Bz[i + j * nb], u[j], acc);
        rr[i] = acc;
      }
      __syncthreads();
      bat_tri_solve(nb, L, Wz, rr, x, bk, xk);
      for (int64_t i = tid; i < nb; i += 256) u[i] += rr[i];
      __syncthreads();
    }
  }
  for (int64_t i = tid; i < nb; i += 256) {
    const double a = i < n ? s * u[i] : 0.0;
    alpha[z * nb + i] = a;
    fhat[z * nb + i] = i < n ? Y[z * nb + i] - sig2 * a : 0.0;
  }
}

// the rows of tmp (64 x ncol, ld NB) back into W (rows k0.., ld nb)
__global__ void bat_copy_rows_kernel(int64_t nb, int64_t k0, int64_t ncol, const double *__restrict__ tmp,
                                     double *__restrict__ W) {
  const int64_t z = blockIdx.y;
  const double *t = tmp + z * NB * nb;
  double *w = W + z * nb * nb;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < NB * ncol;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = idx % NB, c = idx / NB;
    w[k0 + r + c * nb] = t[r + c * NB];
  }
}

__global__ void bat_identity_kernel(int64_t nb, double *__restrict__ W) {
  const int64_t z = blockIdx.y;
  double *w = W + z * nb * nb;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < nb * nb;
       idx += (int64_t)gridDim.x * blockDim.x)
    w[idx] = (idx % nb == idx / nb) ? 1.0 : 0.0;
}

// LML, LOO (with Gauss-Hermite quadrature), prediction mean and variance; one CTA per problem
__global__ void __launch_bounds__(256) bat_finish_kernel(int64_t nb, int64_t mb, const double *__restrict__ prm,
                                                         const int *__restrict__ status,
                                                         const double *__restrict__ Y,
                                                         const double *__restrict__ alpha,
                                                         const double *__restrict__ fhat,
                                                         const double *__restrict__ W,
                                                         const double *__restrict__ ldp,
                                                         const double *__restrict__ R,
                                                         const double *__restrict__ T, int q,
                                                         const double *__restrict__ ghx,
                                                         const double *__restrict__ ghw, double jitter,
                                                         double *__restrict__ lml, double *__restrict__ mean,
                                                         double *__restrict__ var, double *__restrict__ loos,
                                                         double *__restrict__ binv) {
  __shared__ double red[256];
  const int64_t z = blockIdx.x;
  const double *p = prm + z * PRM;
  const int n = (int)p[0], m = (int)p[1];
  const double sig = p[6], sig2 = sig * sig, s = sqrt(1.0 / sig2), m2 = p[5] * p[5];
  const int tid = threadIdx.x;
  if (status[z] != 0) {
    if (tid == 0) lml[z] = -INFINITY;
    return;
  }
  const double *Yz = Y + z * nb, *az = alpha + z * nb, *fz = fhat + z * nb;
  const double *Wz = W + z * nb * nb;
  // diag(B^-1): column norms of W = L^-1, one warp per column
  const int lane = tid & 31, warp = tid >> 5;
  for (int64_t c = warp; c < n; c += 8) {
    double acc = 0.0;
    for (int64_t r = c + lane; r < nb; r += 32) acc = fma(Wz[r + c * nb], Wz[r + c * nb], acc);
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (lane == 0) binv[z * nb + c] = acc;
  }
  // evidence terms: loglik(fhat) - 0.5 fhat^T alpha - sum log L_ii  (R/laplace.R:33-38)
  double acc = 0.0;
  for (int64_t i = tid; i < n; i += 256) {
    const double xx = (Yz[i] - fz[i]) / sig;
    acc += -(0.918938533204672741780329736406 + 0.5 * xx * xx + log(sig)) - 0.5 * fz[i] * az[i];
  }
  red[tid] = acc;
  __syncthreads();
  for (int st = 128; st > 0; st >>= 1) {
    if (tid < st) red[tid] += red[tid + st];
    __syncthreads();
  }
  if (tid == 0) {
    double ld = 0.0;
    for (int64_t k = 0; k < nb / NB; ++k) ld += ldp[z * (nb / NB) + k];
    lml[z] = red[0] - ld;
  }
  __syncthreads();
  // LOO (R/gp_loo.R:119-129, 90-96): post_var = D - D^2 binv / V, D = V + jitter
  for (int64_t i = tid; i < n; i += 256) {
    const double V = sig2, D = V + jitter;
    const double pv = D - D * D * (binv[z * nb + i] / V);
    const double lv = 1.0 / (1.0 / pv - 1.0 / V);
    const double lm = fz[i] - lv * ((Yz[i] - fz[i]) / V);
    const double sd = sqrt(lv);
    double ll[64], mx = -INFINITY;
    for (int k = 0; k < q; ++k) {
      const double f = ghx[k] * sd + lm;
      const double xx = (Yz[i] - f) / sig;
      ll[k] = -(0.918938533204672741780329736406 + 0.5 * xx * xx + log(sig));
      mx = fmax(mx, ll[k]);
    }
    double sacc = 0.0;
    for (int k = 0; k < q; ++k) sacc += ghw[k] * exp(ll[k] - mx);
    loos[z * nb + i] = mx + log(sacc);
  }
  // prediction: mean_j = sum_i K(xt_j, x_i) alpha_i = (R^T alpha)_j / s; var_j = m^2 - |T_j|^2
  const double *Rz = R + z * nb * mb, *Tz = T + z * nb * mb;
  for (int64_t j = warp; j < m; j += 8) {
    double a1 = 0.0, a2 = 0.0;
    for (int64_t i = lane; i < n; i += 32) {
      a1 = fma(Rz[i + j * nb], az[i], a1);
      a2 = fma(Tz[i + j * nb], Tz[i + j * nb], a2);
    }
    for (int o = 16; o > 0; o >>= 1) {
      a1 += __shfl_down_sync(0xffffffffu, a1, o);
      a2 += __shfl_down_sync(0xffffffffu, a2, o);
    }
    if (lane == 0) {
      mean[z * mb + j] = a1 / s;
      var[z * mb + j] = m2 - a2;
    }
  }
}

}  // namespace
}  // namespace gpgp

using namespace gpgp;

struct gpgp_batch {
  gpgp_ctx *ctx = nullptr;
  int precision = 0;
  int quad_order = 11;
  double jitter = 1e-6;
  int32_t nprob = 0;
  std::vector<std::unique_ptr<Bucket>> buckets;
  std::vector<int> bucket_of, slot_of;
  std::vector<gpgp_batch_problem> shape;  // n, d, m of every problem (pointers not kept)
  DBuf ghx, ghw;
  IBuf err;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  double tune_ms[3] = {0, 0, 0};  // autotuning time per variant
  int64_t graph_kernels = 0;  // kernel nodes of the captured graph
  // streams and events of the graph's concurrent bucket lanes (capture only)
  cudaStream_t lanes[4] = {nullptr, nullptr, nullptr, nullptr};
  cudaEvent_t join[4] = {nullptr, nullptr, nullptr, nullptr};
  cudaEvent_t fork = nullptr;
  ~gpgp_batch() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    for (int l = 0; l < 4; ++l) {
      if (lanes[l]) cudaStreamDestroy(lanes[l]);
      if (join[l]) cudaEventDestroy(join[l]);
    }
    if (fork) cudaEventDestroy(fork);
  }
};

namespace {

// The batched problems are small and smooth: their B has entries of nearly equal
// size, so the 32-bit slices of the factorisation path leave log-determinant
// errors near 1e-6. Five slices (40-bit) and two FP64 refinement steps of alpha
// bring the evidence to ~1e-9.
constexpr int kSlices = 5;
constexpr int kRefine = 2;

size_t split_stride_bytes(int64_t rows, int64_t K) {
  return (oz_split_bytes(rows, K, kSlices) + 1023) / 1024 * 1024;
}

// one bucket's pipeline, enqueued on stream st (no allocation, no sync)
void run_bucket(gpgp_batch *b, Bucket &k, cudaStream_t st) {
  const int64_t nb = k.nb, mb = k.mb, P = k.count, nbl = nb / NB;
  GPGP_CUDA(cudaMemsetAsync(k.status.p, 0, P * sizeof(int), st));
  {
    const int64_t T = nb / BT;
    dim3 g((unsigned)(T * (T + 1) / 2), (unsigned)P);
    if (b->precision == GPGP_PREC_MIXED)
      bat_cov_B_kernel<true><<<g, 256, 0, st>>>(nb, k.dm, k.X.p, k.prm.p, b->jitter, k.Bm.p,
                                                k.variant >= 1 ? k.Bc.p : nullptr);
    else
      bat_cov_B_kernel<false><<<g, 256, 0, st>>>(nb, k.dm, k.X.p, k.prm.p, b->jitter, k.Bm.p,
                                                 k.variant >= 1 ? k.Bc.p : nullptr);
    GPGP_CHECK_LAUNCH();
  }
  {
    dim3 g((unsigned)(nb / BT), (unsigned)((mb + BT - 1) / BT), (unsigned)P);
    if (b->precision == GPGP_PREC_MIXED)
      bat_cross_kernel<true><<<g, 256, 0, st>>>(nb, mb, k.dm, k.X.p, k.Xt.p, k.prm.p, k.R.p);
    else
      bat_cross_kernel<false><<<g, 256, 0, st>>>(nb, mb, k.dm, k.X.p, k.Xt.p, k.prm.p, k.R.p);
    GPGP_CHECK_LAUNCH();
  }
  // Cholesky of B
  if (k.variant == 0) {
    potrf_batched(st, k.Bm.p, nb, nb, nb * nb, k.Winv.p, nb * NB, k.ldp.p, nbl, k.status.p, P);
  } else {
    // tensor variants: outer panels of 64 (variant 1: a trailing update after every
    // diagonal block, K = 64) or 256 columns (variant 2: the panel's blocks update
    // the rest of the panel, then one trailing update with K = 256)
    const int64_t outer = k.variant == 2 ? 4 * NB : NB;
    for (int64_t k0 = 0; k0 < nb; k0 += outer) {
      const int64_t kbo = std::min<int64_t>(outer, nb - k0);
      for (int64_t j0 = k0; j0 < k0 + kbo; j0 += NB) {
        const int64_t blk = j0 / NB;
        double *Akk = k.Bm.p + j0 + j0 * nb;
        {
          KTScope kts(GPGP_KPROF_POTRF_DIAG, st, 2.0 * NB * NB * NB / 3 * (double)P);
          potrf_diag_kernel<<<(unsigned)P, DIAG_THREADS, 0, st>>>(Akk, NB, nb, k.Winv.p + blk * NB * NB,
                                                                  k.ldp.p + blk, k.status.p, j0, nb * nb, nb * NB,
                                                                  nbl);
        }
        GPGP_CHECK_LAUNCH();
        const int64_t m = nb - j0 - NB;
        if (m <= 0) continue;
        double *A21 = k.Bm.p + (j0 + NB) + j0 * nb;
        // L21 = A21 W^T
        oz_split_batched(st, A21, nb, nb * nb, 0, m, NB, &k.SA, P);
        oz_split_batched(st, k.Winv.p + blk * NB * NB, NB, nb * NB, 0, NB, NB, &k.SB, P);
        oz_gemm_batched(st, k.SA, 0, k.SB, 0, m, NB, 0, 1, 0, 1.0, 0.0, A21, nb, nb * nb, false, b->err.p,
                        k.status.p, 1, P);
        // the rest of this outer panel's columns
        const int64_t nc = k0 + kbo - (j0 + NB);
        if (nc > 0) {
          oz_split_batched(st, A21, nb, nb * nb, 0, m, NB, &k.SA, P);
          oz_gemm_batched(st, k.SA, 0, k.SA, 0, m, nc, 0, 1, 0, -1.0, 1.0, k.Bm.p + (j0 + NB) * (1 + nb), nb,
                          nb * nb, true, b->err.p, k.status.p, 1, P);
        }
      }
      // trailing update with the finished outer panel
      const int64_t m2 = nb - k0 - kbo;
      if (m2 <= 0) continue;
      oz_split_batched(st, k.Bm.p + (k0 + kbo) + k0 * nb, nb, nb * nb, 0, m2, kbo, &k.SA, P);
      oz_gemm_batched(st, k.SA, 0, k.SA, 0, m2, m2, 0, kbo / NB, 0, -1.0, 1.0, k.Bm.p + (k0 + kbo) * (1 + nb), nb,
                      nb * nb, true, b->err.p, k.status.p, 1, P);
    }
  }
  bat_solve_kernel<<<(unsigned)P, 256, 0, st>>>(nb, k.Bm.p, k.Winv.p, k.variant >= 1 ? k.Bc.p : nullptr,
                                                kRefine, k.Y.p, k.prm.p, k.status.p, k.tmp.p, k.tmp.p + P * nb,
                                                k.tmp.p + 2 * P * nb, k.alpha.p, k.fhat.p);
  GPGP_CHECK_LAUNCH();
  // W = L^-1: blocked solve against I (R/gp_loo.R needs diag(B^-1), prediction needs W R)
  {
    dim3 g((unsigned)std::min<int64_t>((nb * nb + 255) / 256, 1024), (unsigned)P);
    bat_identity_kernel<<<g, 256, 0, st>>>(nb, k.W.p);
    GPGP_CHECK_LAUNCH();
  }
  for (int64_t k0 = 0, blk = 0; k0 < nb; k0 += NB, ++blk) {
    const int64_t ncol = k0 + NB;
    gemm64_batched(st, false, false, NB, ncol, NB, 1.0, k.Winv.p + blk * NB * NB, NB, nb * NB, k.W.p + k0, nb,
                   nb * nb, 0.0, k.tmp.p, NB, NB * nb, P);
    dim3 g((unsigned)std::min<int64_t>((NB * ncol + 255) / 256, 256), (unsigned)P);
    bat_copy_rows_kernel<<<g, 256, 0, st>>>(nb, k0, ncol, k.tmp.p, k.W.p);
    GPGP_CHECK_LAUNCH();
    const int64_t rest = nb - ncol;
    if (rest <= 0) continue;
    if (k.variant == 0) {
      gemm64_batched(st, false, false, rest, ncol, NB, -1.0, k.Bm.p + ncol + k0 * nb, nb, nb * nb, k.tmp.p,
                     NB, NB * nb, 1.0, k.W.p + ncol, nb, nb * nb, P);
    } else {
      oz_split_batched(st, k.Bm.p + ncol + k0 * nb, nb, nb * nb, 0, rest, NB, &k.SA, P);
      oz_split_batched(st, k.tmp.p, NB, NB * nb, 1, ncol, NB, &k.SB, P);
      oz_gemm_batched(st, k.SA, 0, k.SB, 0, rest, ncol, 0, 1, 0, -1.0, 1.0, k.W.p + ncol, nb, nb * nb, false,
                      b->err.p, nullptr, 0, P);
    }
  }
  // T = W R (prediction variance)
  if (k.variant == 0) {
    gemm64_batched(st, false, false, nb, mb, nb, 1.0, k.W.p, nb, nb * nb, k.R.p, nb, nb * mb, 0.0, k.T.p, nb,
                   nb * mb, P);
  } else {
    oz_split_batched(st, k.W.p, nb, nb * nb, 0, nb, nb, &k.SA, P);
    oz_split_batched(st, k.R.p, nb, nb * mb, 1, mb, nb, &k.SB, P);
    oz_gemm_batched(st, k.SA, 0, k.SB, 0, nb, mb, 0, k.SA.nkb, 3, 1.0, 0.0, k.T.p, nb, nb * mb, false,
                    b->err.p, nullptr, 0, P);
  }
  bat_finish_kernel<<<(unsigned)P, 256, 0, st>>>(nb, mb, k.prm.p, k.status.p, k.Y.p, k.alpha.p, k.fhat.p, k.W.p,
                                                 k.ldp.p, k.R.p, k.T.p, b->quad_order, b->ghx.p, b->ghw.p,
                                                 b->jitter, k.lml.p, k.mean.p, k.var.p, k.loos.p, k.binv.p);
  GPGP_CHECK_LAUNCH();
}

void run_all(gpgp_batch *b) {
  for (auto &k : b->buckets) run_bucket(b, *k, b->ctx->stream);
}

// The buckets share nothing but the read-only quadrature nodes and the error word
// (set, never cleared, by the kernels), so they can run side by side: the graph
// forks from the context stream into up to kLanes streams, each running its
// buckets in turn, and joins back. Buckets go to lanes longest first by their
// measured time (the autotuner's; FP64 plans: count x nb^3), each to the lane
// with the least work so far. Small buckets whose launches fill few SMs then
// overlap with the large ones.
constexpr int kLanes = 4;

void run_all_lanes(gpgp_batch *b) {
  cudaStream_t st = b->ctx->stream;
  const int nl = std::min<int>(kLanes, (int)b->buckets.size());
  if (nl <= 1) return run_all(b);
  std::vector<int> order(b->buckets.size());
  for (size_t i = 0; i < order.size(); ++i) order[i] = (int)i;
  auto cost = [&](int i) {
    const Bucket &k = *b->buckets[i];
    return k.best_ms > 0 ? k.best_ms : (double)k.count * k.nb * k.nb * k.nb;
  };
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return cost(x) > cost(y); });
  std::vector<double> load(nl, 0.0);
  std::vector<std::vector<int>> lane(nl);
  for (int i : order) {
    const int l = (int)(std::min_element(load.begin(), load.end()) - load.begin());
    lane[l].push_back(i);
    load[l] += cost(i);
  }
  GPGP_CUDA(cudaEventRecord(b->fork, st));
  for (int l = 0; l < nl; ++l) {
    GPGP_CUDA(cudaStreamWaitEvent(b->lanes[l], b->fork, 0));
    for (int i : lane[l]) run_bucket(b, *b->buckets[i], b->lanes[l]);
    GPGP_CUDA(cudaEventRecord(b->join[l], b->lanes[l]));
    GPGP_CUDA(cudaStreamWaitEvent(st, b->join[l], 0));
  }
}

// copy the inputs of every problem into its bucket slot (host buffers)
void upload(gpgp_batch *b, const gpgp_batch_problem *probs) {
  cudaStream_t st = b->ctx->stream;
  for (auto &kp : b->buckets) {
    Bucket &k = *kp;
    std::vector<double> prm(k.count * PRM, 0.0), X(k.count * k.nb * k.dm, 0.0), Y(k.count * k.nb, 0.0),
        Xt(k.count * k.mb * k.dm, 0.0);
    for (int64_t s = 0; s < k.count; ++s) {
      const gpgp_batch_problem &p = probs[k.probs[s]];
      double *pp = &prm[s * PRM];
      pp[0] = p.n;
      pp[1] = p.m;
      pp[2] = p.d;
      pp[3] = p.kind;
      pp[4] = p.lscale;
      pp[5] = p.magn;
      pp[6] = p.sigma;
      for (int64_t c = 0; c < p.d; ++c) {
        for (int64_t i = 0; i < p.n; ++i) X[s * k.nb * k.dm + c * k.nb + i] = p.x[i + c * p.n];
        for (int64_t j = 0; j < p.m; ++j) Xt[s * k.mb * k.dm + c * k.mb + j] = p.xt[j + c * p.m];
      }
      for (int64_t i = 0; i < p.n; ++i) Y[s * k.nb + i] = p.y[i];
    }
    GPGP_CUDA(cudaMemcpyAsync(k.prm.p, prm.data(), prm.size() * 8, cudaMemcpyHostToDevice, st));
    GPGP_CUDA(cudaMemcpyAsync(k.X.p, X.data(), X.size() * 8, cudaMemcpyHostToDevice, st));
    GPGP_CUDA(cudaMemcpyAsync(k.Y.p, Y.data(), Y.size() * 8, cudaMemcpyHostToDevice, st));
    GPGP_CUDA(cudaMemcpyAsync(k.Xt.p, Xt.data(), Xt.size() * 8, cudaMemcpyHostToDevice, st));
    GPGP_CUDA(cudaStreamSynchronize(st));
  }
}

std::string check_problems(const gpgp_batch_problem *probs, int32_t nprob) {
  for (int32_t i = 0; i < nprob; ++i) {
    const gpgp_batch_problem &p = probs[i];
    if (p.n < 1 || p.n > 4096 || p.d < 1 || p.d > 8 || p.m < 0 || !p.x || !p.y || (p.m > 0 && !p.xt) ||
        !(p.sigma > 0) || !(p.lscale > 0) ||
        (p.kind != GPGP_CF_SEXP && p.kind != GPGP_CF_MATERN32 && p.kind != GPGP_CF_MATERN52))
      return "batched problem " + std::to_string(i) + " is invalid";
    bool finite = true;
    for (int64_t k = 0; k < (int64_t)p.n * p.d && finite; ++k) finite = std::isfinite(p.x[k]);
    for (int64_t k = 0; k < p.n && finite; ++k) finite = std::isfinite(p.y[k]);
    for (int64_t k = 0; k < (int64_t)p.m * p.d && finite; ++k) finite = std::isfinite(p.xt[k]);
    if (!finite) return "batched problem " + std::to_string(i) + " holds NaN or Inf";
  }
  return std::string();
}

// buckets, device buffers and the first upload of a plan
void build_plan(gpgp_batch *b, gpgp_ctx *ctx, const gpgp_batch_problem *probs, int32_t nprob,
                int32_t precision, int32_t quad_order, double jitter) {
  GPGP_CUDA(cudaSetDevice(ctx->device));
  b->ctx = ctx;
  b->precision = precision;
  b->quad_order = quad_order;
  b->jitter = jitter;
  b->nprob = nprob;
  b->shape.assign(probs, probs + nprob);
  cudaStream_t st = ctx->stream;
  std::map<int64_t, std::vector<int>> groups;
  for (int32_t i = 0; i < nprob; ++i) groups[(probs[i].n + NB - 1) / NB * NB].push_back(i);
  b->bucket_of.assign(nprob, 0);
  b->slot_of.assign(nprob, 0);
  for (auto &g : groups) {
    std::unique_ptr<Bucket> k(new Bucket());
    k->nb = g.first;
    k->count = (int64_t)g.second.size();
    k->probs = g.second;
    int64_t mb = 1, dm = 1;
    for (int i : g.second) {
      mb = std::max<int64_t>(mb, probs[i].m);
      dm = std::max<int64_t>(dm, probs[i].d);
    }
    k->mb = (mb + NB - 1) / NB * NB;
    k->dm = dm;
    const int64_t P = k->count, nb = k->nb, mbb = k->mb;
    k->prm.alloc(st, P * PRM);
    k->X.alloc(st, P * nb * dm);
    k->Y.alloc(st, P * nb);
    k->Xt.alloc(st, P * mbb * dm);
    k->Bm.alloc(st, P * nb * nb);
    k->Winv.alloc(st, P * nb * NB);
    k->ldp.alloc(st, P * (nb / NB));
    k->W.alloc(st, P * nb * nb);
    k->R.alloc(st, P * nb * mbb);
    k->T.alloc(st, P * nb * mbb);
    k->tmp.alloc(st, std::max<int64_t>(P * NB * nb, 3 * P * nb));
    k->alpha.alloc(st, P * nb);
    k->fhat.alloc(st, P * nb);
    k->lml.alloc(st, P);
    k->mean.alloc(st, P * mbb);
    k->var.alloc(st, P * mbb);
    k->loos.alloc(st, P * nb);
    k->binv.alloc(st, P * nb);
    k->status.alloc(st, P);
    if (precision == GPGP_PREC_MIXED) {
      // per-problem sliced operands: at most nb rows x nb K (A), max(nb, mb) rows x nb K (B)
      const size_t ba = split_stride_bytes(nb, nb), bb = split_stride_bytes(std::max(nb, mbb), nb);
      if (cudaMallocAsync(&k->sa, ba * P, st) != cudaSuccess || cudaMallocAsync(&k->sb, bb * P, st) != cudaSuccess) {
        (void)cudaGetLastError();
        throw std::bad_alloc();
      }
      oz_split_bind(k->sa, nb, nb, &k->SA, kSlices);
      oz_split_bind(k->sb, std::max(nb, mbb), nb, &k->SB, kSlices);
      k->Bc.alloc(st, P * nb * nb);
      // batch strides in elements of each array (ex ints, slices uint16)
      k->SA.bstride_ex = (int64_t)(ba / sizeof(int));
      k->SA.bstride_sl = (int64_t)(ba / sizeof(uint16_t));
      k->SB.bstride_ex = (int64_t)(bb / sizeof(int));
      k->SB.bstride_sl = (int64_t)(bb / sizeof(uint16_t));
    }
    k->variant = precision == GPGP_PREC_MIXED ? 1 : 0;
    for (int64_t s = 0; s < P; ++s) {
      b->bucket_of[g.second[s]] = (int)b->buckets.size();
      b->slot_of[g.second[s]] = (int)s;
    }
    b->buckets.push_back(std::move(k));
  }
  std::vector<double> hx, hw;
  gauss_hermite(quad_order, &hx, &hw);
  copy_in(st, b->ghx, hx.data(), quad_order, false);
  copy_in(st, b->ghw, hw.data(), quad_order, false);
  b->err.alloc(st, 1);
  GPGP_CUDA(cudaMemsetAsync(b->err.p, 0, sizeof(int), st));
  upload(b, probs);
}

}  // namespace

// One-shot batched solve for the request server: plan, upload, run the pipeline
// once without autotuning or graph capture (the tensor-core variant for mixed
// precision, the FP64 pipe otherwise, so a problem's result does not depend on
// its batch-mates) and read the evidence, predictive means and variances back.
gpgp_status gpgp::batch_solve_once(gpgp_ctx *ctx, const gpgp_batch_problem *probs, int32_t nprob,
                                   int32_t precision, double jitter, double *lml, double *mean,
                                   double *var) {
  if (std::string why = check_problems(probs, nprob); !why.empty()) return fail(ctx, GPGP_EINVAL, why);
  gpgp_status st = guarded(ctx, [&]() -> gpgp_status {
    gpgp_batch b;
    build_plan(&b, ctx, probs, nprob, precision, 11, jitter);
    run_all(&b);
    return gpgp_batch_results(&b, lml, mean, var, nullptr);
  });
  return st;
}

// Device bytes of a one-shot batch holding one problem of this size (the
// allocations of build_plan, rounded up per problem).
size_t gpgp::batch_bytes_estimate(int64_t n, int64_t m, int32_t d, int32_t precision) {
  const int64_t nb = (n + NB - 1) / NB * NB, mb = std::max<int64_t>(NB, (m + NB - 1) / NB * NB);
  size_t b = 8 * (size_t)(PRM + nb * d + nb + mb * d + 2 * nb * nb + nb * NB + nb / NB + 2 * nb * mb +
                          std::max<int64_t>(NB * nb, 3 * nb) + 4 * nb + 1 + 2 * mb) + 4;
  if (precision == GPGP_PREC_MIXED)
    b += 8 * (size_t)nb * nb + split_stride_bytes(nb, nb) + split_stride_bytes(std::max(nb, mb), nb);
  return b;
}

extern "C" {

gpgp_status gpgp_batch_create(gpgp_ctx *ctx, const gpgp_batch_problem *probs, int32_t nprob,
                              int32_t precision, int32_t quad_order, double jitter, gpgp_batch **out) {
  if (!ctx || !probs || nprob < 1 || !out || quad_order < 1 || quad_order > 64)
    return fail(ctx, GPGP_EINVAL, "invalid argument");
  *out = nullptr;
  if (std::string why = check_problems(probs, nprob); !why.empty()) return fail(ctx, GPGP_EINVAL, why);
  return guarded(ctx, [&]() -> gpgp_status {
    std::unique_ptr<gpgp_batch> b(new gpgp_batch());
    build_plan(b.get(), ctx, probs, nprob, precision, quad_order, jitter);
    cudaStream_t st = ctx->stream;
    // autotune: the FP64 pipe or the sliced tensor-core GEMM, per bucket (mixed precision only)
    cudaEvent_t e0, e1;
    GPGP_CUDA(cudaEventCreate(&e0));
    GPGP_CUDA(cudaEventCreate(&e1));
    for (auto &kp : b->buckets) {
      Bucket &k = *kp;
      const int nvar = precision == GPGP_PREC_MIXED ? 3 : 1;
      float best = 1e30f;
      int bestv = 0;
      for (int v = 0; v < nvar; ++v) {
        k.variant = v;
        run_bucket(b.get(), k, st);  // warm
        GPGP_CUDA(cudaEventRecord(e0, st));
        run_bucket(b.get(), k, st);
        GPGP_CUDA(cudaEventRecord(e1, st));
        GPGP_CUDA(cudaEventSynchronize(e1));
        float ms = 0.f;
        GPGP_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        b->tune_ms[v] += ms;
        if (ms < best) {
          best = ms;
          bestv = v;
        }
      }
      k.variant = bestv;
      k.best_ms = nvar > 1 ? best : 0.0;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    for (int l = 0; l < kLanes; ++l) {
      GPGP_CUDA(cudaStreamCreateWithFlags(&b->lanes[l], cudaStreamNonBlocking));
      GPGP_CUDA(cudaEventCreateWithFlags(&b->join[l], cudaEventDisableTiming));
    }
    GPGP_CUDA(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming));
    // capture the whole pipeline once; the graph's kernel nodes are counted per replay
    GPGP_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    tl_capturing = true;
    try {
      run_all_lanes(b.get());
    } catch (...) {
      tl_capturing = false;
      cudaGraph_t g = nullptr;
      cudaStreamEndCapture(st, &g);
      if (g) cudaGraphDestroy(g);
      throw;
    }
    tl_capturing = false;
    GPGP_CUDA(cudaStreamEndCapture(st, &b->graph));
    size_t nnodes = 0;
    GPGP_CUDA(cudaGraphGetNodes(b->graph, nullptr, &nnodes));
    std::vector<cudaGraphNode_t> nodes(nnodes);
    if (nnodes) GPGP_CUDA(cudaGraphGetNodes(b->graph, nodes.data(), &nnodes));
    for (auto nd : nodes) {
      cudaGraphNodeType ty;
      GPGP_CUDA(cudaGraphNodeGetType(nd, &ty));
      if (ty == cudaGraphNodeTypeKernel) ++b->graph_kernels;
    }
    GPGP_CUDA(cudaGraphInstantiate(&b->exec, b->graph, 0));
    *out = b.release();
    return GPGP_OK;
  });
}

gpgp_status gpgp_batch_run(gpgp_batch *b) {
  if (!b) return GPGP_EINVAL;
  return guarded(b->ctx, [&]() -> gpgp_status {
    GPGP_CUDA(cudaGraphLaunch(b->exec, b->ctx->stream));
    g_launches += b->graph_kernels;
    return GPGP_OK;
  });
}

gpgp_status gpgp_batch_upload(gpgp_batch *b, const gpgp_batch_problem *probs) {
  if (!b || !probs) return GPGP_EINVAL;
  for (int32_t i = 0; i < b->nprob; ++i)
    if (probs[i].n != b->shape[i].n || probs[i].d != b->shape[i].d || probs[i].m != b->shape[i].m)
      return fail(b->ctx, GPGP_EINVAL, "gpgp_batch_upload: problem shapes differ from the plan");
  return guarded(b->ctx, [&]() -> gpgp_status {
    upload(b, probs);
    return GPGP_OK;
  });
}

gpgp_status gpgp_batch_results(gpgp_batch *b, double *log_evidence, double *mean, double *var,
                               double *loos) {
  if (!b) return GPGP_EINVAL;
  return guarded(b->ctx, [&]() -> gpgp_status {
    cudaStream_t st = b->ctx->stream;
    std::vector<std::vector<double>> hl(b->buckets.size()), hm(b->buckets.size()), hv(b->buckets.size()),
        ho(b->buckets.size());
    for (size_t g = 0; g < b->buckets.size(); ++g) {
      Bucket &k = *b->buckets[g];
      hl[g].resize(k.count);
      GPGP_CUDA(cudaMemcpyAsync(hl[g].data(), k.lml.p, k.count * 8, cudaMemcpyDeviceToHost, st));
      if (mean) {
        hm[g].resize(k.count * k.mb);
        GPGP_CUDA(cudaMemcpyAsync(hm[g].data(), k.mean.p, hm[g].size() * 8, cudaMemcpyDeviceToHost, st));
      }
      if (var) {
        hv[g].resize(k.count * k.mb);
        GPGP_CUDA(cudaMemcpyAsync(hv[g].data(), k.var.p, hv[g].size() * 8, cudaMemcpyDeviceToHost, st));
      }
      if (loos) {
        ho[g].resize(k.count * k.nb);
        GPGP_CUDA(cudaMemcpyAsync(ho[g].data(), k.loos.p, ho[g].size() * 8, cudaMemcpyDeviceToHost, st));
      }
    }
    int herr = 0;
    GPGP_CUDA(cudaMemcpyAsync(&herr, b->err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    GPGP_CUDA(cudaStreamSynchronize(st));
    if (herr) return fail(b->ctx, GPGP_ETIMEOUT, "a tensor-core kernel wait timed out");
    // outputs are packed per problem in input order: mean/var m_i values, loos n_i values
    int64_t om = 0, oo = 0;
    for (int32_t i = 0; i < b->nprob; ++i) {
      const int g = b->bucket_of[i], s = b->slot_of[i];
      const Bucket &k = *b->buckets[g];
      if (log_evidence) log_evidence[i] = hl[g][s];
      const int64_t m = b->shape[i].m, n = b->shape[i].n;
      if (mean)
        for (int64_t j = 0; j < m; ++j) mean[om + j] = hm[g][s * k.mb + j];
      if (var)
        for (int64_t j = 0; j < m; ++j) var[om + j] = hv[g][s * k.mb + j];
      if (loos)
        for (int64_t j = 0; j < n; ++j) loos[oo + j] = ho[g][s * k.nb + j];
      om += m;
      oo += n;
    }
    return GPGP_OK;
  });
}

gpgp_status gpgp_batch_info(gpgp_batch *b, int32_t *nbuckets, int32_t *bucket_n, int32_t *bucket_count,
                            int32_t *bucket_variant, double *tune_ms) {
  if (!b) return GPGP_EINVAL;
  if (nbuckets) *nbuckets = (int32_t)b->buckets.size();
  for (size_t g = 0; g < b->buckets.size(); ++g) {
    if (bucket_n) bucket_n[g] = (int32_t)b->buckets[g]->nb;
    if (bucket_count) bucket_count[g] = (int32_t)b->buckets[g]->count;
    if (bucket_variant) bucket_variant[g] = b->buckets[g]->variant;
  }
  if (tune_ms)
    for (int v = 0; v < 3; ++v) tune_ms[v] = b->tune_ms[v];
  return GPGP_OK;
}

gpgp_status gpgp_batch_destroy(gpgp_batch *b) {
  if (!b) return GPGP_OK;
  cudaSetDevice(b->ctx->device);
  cudaStreamSynchronize(b->ctx->stream);
  delete b;
  return GPGP_OK;
}

}  // extern "C"
