// k-means for FITC's inducing inputs (get_inducing, R/gp_fit.R:192-236).
//
// The reference runs stats::kmeans (Hartigan-Wong, random initial centres from
// R's stream) on the standardised inputs. Neither R's stream nor its algorithm
// can be reproduced here, so this is Lloyd's algorithm from caller-given
// initial centres, with the same iteration limit: every point goes to its
// nearest centre (squared distance, ties to the lower index), every centre to
// the mean of its points (an empty cluster keeps its centre). The centre sums
// are deterministic: each block sums its chunk of points per cluster in point
// order, and the block partials are added in block order.
#include <math.h>

#include <algorithm>
#include <vector>

#include "common.cuh"
#include "model.cuh"

namespace gpgp {
namespace {

constexpr int KM_CHUNK = 256;  // points per block in the centre sums

// nearest centre of every point; x is n x d column-major, centres k x d
__global__ void km_assign_kernel(const double *__restrict__ x, int64_t n, int d, const double *__restrict__ c,
                                 int k, int *__restrict__ assign, int *__restrict__ changed,
                                 double *__restrict__ wss_part) {
  extern __shared__ double cs[];  // k x d
  for (int idx = threadIdx.x; idx < k * d; idx += blockDim.x) cs[idx] = c[idx];
  __syncthreads();
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  double best = INFINITY;
  if (i < n) {
    int bj = 0;
    for (int j = 0; j < k; ++j) {
      double s = 0.0;
      for (int t = 0; t < d; ++t) {
        const double df = x[i + t * n] - cs[j + t * k];
        s = fma(df, df, s);
      }
      if (s < best) {
        best = s;
        bj = j;
      }
    }
    if (assign[i] != bj) {
      assign[i] = bj;
      *changed = 1;
    }
  }
  // block sum of the squared distances (fixed tree order)
  __shared__ double red[256];
  red[threadIdx.x] = i < n ? best : 0.0;
  __syncthreads();
  for (int st = blockDim.x / 2; st > 0; st >>= 1) {
    if (threadIdx.x < st) red[threadIdx.x] += red[threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x == 0) wss_part[blockIdx.x] = red[0];
}

// per block: for its chunk of points, thread j sums the points of clusters
// j, j + blockDim, ... in point order -> part[block][cluster][0..d-1], count at [d]
__global__ void km_partial_kernel(const double *__restrict__ x, int64_t n, int d, const int *__restrict__ assign,
                                  int k, double *__restrict__ part) {
  const int64_t p0 = (int64_t)blockIdx.x * KM_CHUNK;
  const int64_t p1 = p0 + KM_CHUNK < n ? p0 + KM_CHUNK : n;
  __shared__ int as[KM_CHUNK];
  for (int64_t p = p0 + threadIdx.x; p < p1; p += blockDim.x) as[p - p0] = assign[p];
  __syncthreads();
  double *out = part + (int64_t)blockIdx.x * k * (d + 1);
  for (int j = threadIdx.x; j < k; j += blockDim.x) {
    double cnt = 0.0;
    double acc[16];
    for (int t = 0; t < d; ++t) acc[t] = 0.0;
    for (int64_t p = p0; p < p1; ++p)
      if (as[p - p0] == j) {
        cnt += 1.0;
        for (int t = 0; t < d; ++t) acc[t] += x[p + t * n];
      }
    for (int t = 0; t < d; ++t) out[j * (d + 1) + t] = acc[t];
    out[j * (d + 1) + d] = cnt;
  }
}

// centres = sums / counts over the blocks in order; an empty cluster keeps its centre
__global__ void km_update_kernel(const double *__restrict__ part, int nblocks, int d, int k, double *__restrict__ c) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= k) return;
  double cnt = 0.0, acc[16];
  for (int t = 0; t < d; ++t) acc[t] = 0.0;
  for (int b = 0; b < nblocks; ++b) {
    const double *q = part + ((int64_t)b * k + j) * (d + 1);
    for (int t = 0; t < d; ++t) acc[t] += q[t];
    cnt += q[d];
  }
  if (cnt > 0.0)
    for (int t = 0; t < d; ++t) c[j + t * k] = acc[t] / cnt;
}

}  // namespace
}  // namespace gpgp

using namespace gpgp;

extern "C" gpgp_status gpgp_kmeans(gpgp_ctx *ctx, const double *x, int64_t n, int32_t d, int32_t k,
                                   const double *init, int32_t max_iter, double *centers, int32_t *iters,
                                   double *wss) {
  if (!ctx || !x || !init || !centers || n < 1 || d < 1 || d > 16 || k < 1 || k > n || max_iter < 1 ||
      (int64_t)k * d > 6144)
    return fail(ctx, GPGP_EINVAL, "invalid argument (d <= 16, k <= n, k d <= 6144)");
  return guarded(ctx, [&]() -> gpgp_status {
    GPGP_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    DBuf dx, dc, part, wpart;
    IBuf assign, changed;
    copy_in(s, dx, x, (size_t)n * d, false);
    copy_in(s, dc, init, (size_t)k * d, false);
    assign.alloc(s, n);
    GPGP_CUDA(cudaMemsetAsync(assign.p, 0xff, n * sizeof(int), s));  // -1: every point changes at first
    changed.alloc(s, 1);
    const unsigned ablocks = (unsigned)((n + 255) / 256);
    const int pblocks = (int)((n + KM_CHUNK - 1) / KM_CHUNK);
    part.alloc(s, (size_t)pblocks * k * (d + 1));
    wpart.alloc(s, ablocks);
    const size_t smem = (size_t)k * d * sizeof(double);
    if (smem > 48 * 1024)
      GPGP_CUDA(cudaFuncSetAttribute(km_assign_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int it = 0;
    for (it = 1; it <= max_iter; ++it) {
      GPGP_CUDA(cudaMemsetAsync(changed.p, 0, sizeof(int), s));
      km_assign_kernel<<<ablocks, 256, smem, s>>>(dx.p, n, d, dc.p, k, assign.p, changed.p, wpart.p);
      GPGP_CHECK_LAUNCH();
      int hc = 0;
      GPGP_CUDA(cudaMemcpyAsync(&hc, changed.p, sizeof(int), cudaMemcpyDeviceToHost, s));
      GPGP_CUDA(cudaStreamSynchronize(s));
      if (!hc) break;  // converged: the centres are the means of the current clusters
      km_partial_kernel<<<(unsigned)pblocks, 256, 0, s>>>(dx.p, n, d, assign.p, k, part.p);
      GPGP_CHECK_LAUNCH();
      km_update_kernel<<<(unsigned)((k + 127) / 128), 128, 0, s>>>(part.p, pblocks, d, k, dc.p);
      GPGP_CHECK_LAUNCH();
    }
    if (it > max_iter) it = max_iter;
    if (iters) *iters = it;
    if (wss) {
      // within-cluster sum of squares of the final centres
      km_assign_kernel<<<ablocks, 256, smem, s>>>(dx.p, n, d, dc.p, k, assign.p, changed.p, wpart.p);
      GPGP_CHECK_LAUNCH();
      std::vector<double> hw(ablocks);
      GPGP_CUDA(cudaMemcpyAsync(hw.data(), wpart.p, ablocks * sizeof(double), cudaMemcpyDeviceToHost, s));
      GPGP_CUDA(cudaStreamSynchronize(s));
      double t = 0.0;
      for (double v : hw) t += v;
      *wss = t;
    }
    GPGP_CUDA(cudaMemcpyAsync(centers, dc.p, (size_t)k * d * sizeof(double), cudaMemcpyDeviceToHost, s));
    GPGP_CUDA(cudaStreamSynchronize(s));
    return GPGP_OK;
  });
}
