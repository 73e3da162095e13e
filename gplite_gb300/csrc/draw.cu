// Posterior predictive covariance and multivariate normal draws (gp_draw).
//
// gp_draw (R/gp_draw.R:1-143) takes the predictive covariance of
// gp_pred_post(cov = TRUE) (R/gp_pred.R:202-232):
//   cov = K(xt, xt) - aux^T aux + jitter I,   aux = C_chol^-1 K(x, xt)
// and draws mean + t(chol(cov)) Z (mvnrnd, R/gp_draw.R:182-199). Both steps run
// here on the device in FP64: the covariance from the model's resident factor
// (blocked solve + one FP64 GEMM), the draws from a Cholesky of the covariance
// and one GEMM. The standard-normal matrix Z is the caller's, so a draw is a
// deterministic function of it.
#include <math.h>

#include <algorithm>

#include "common.cuh"
#include "model.cuh"

namespace gpgp {
namespace {

__global__ void add_diag_kernel(double *__restrict__ C, int64_t n, int64_t ldc, double v) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) C[i + i * ldc] += v;
}

__global__ void zero_upper_cols_kernel(double *__restrict__ C, int64_t n, int64_t ldc) {
  for (int64_t j = blockIdx.y; j < n; j += gridDim.y)
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < j; i += (int64_t)gridDim.x * blockDim.x)
      C[i + j * ldc] = 0.0;
}

__global__ void broadcast_cols_kernel(const double *__restrict__ v, int64_t d, int64_t cols, double *__restrict__ out) {
  const int64_t total = d * cols;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x)
    out[idx] = v[idx % d];
}

}  // namespace
}  // namespace gpgp

using namespace gpgp;

extern "C" {

gpgp_status gpgp_pred_cov(gpgp_model *m, const double *xt, int64_t mt, uint32_t group_mask, double jitter,
                          double *mean, double *cov) {
  if (!m || !xt || !mean || !cov || mt < 1) return fail(m ? m->ctx : nullptr, GPGP_EINVAL, "invalid argument");
  if (!m->fitted) return fail(m->ctx, GPGP_ENOT_FITTED, "model is not fitted");
  if (m->nlc || m->improper)
    return fail(m->ctx, GPGP_EUNSUPPORTED, "predictive covariance of a non-log-concave fit is not available");
  if (m->rf)
    return fail(m->ctx, GPGP_EUNSUPPORTED,
                "method_rf / method_rbf have no predictive covariance (gp_pred_post.method_rf has no cov); "
                "draw in weight space with gpgp_rf_draw");
  gpgp_ctx *ctx = m->ctx;
  return guarded(ctx, [&]() -> gpgp_status {
    GPGP_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    const int64_t n = m->n;
    const uint32_t gm = group_mask ? group_mask : 0xffffffffu;
    DBuf dxt, Ft, dmean, C, R, tmp;
    IBuf status;
    copy_in(s, dxt, xt, (size_t)mt * m->d, false);
    Ft.alloc(s, (size_t)mt * std::max(1, m->dk.nfeat));
    prep_features(s, m->dk, m->prep, dxt.p, mt, mt, Ft.p, mt);
    dmean.alloc(s, mt);
    if (m->fitc) {  // gp_pred_post.method_fitc(cov = TRUE), R/gp_pred.R:263-276
      C.alloc(s, (size_t)mt * mt);
      gpgp_status st = pred_cov_fitc(m, Ft.p, mt, gm, jitter, dmean.p, C.p);
      if (st != GPGP_OK) return st;
      GPGP_CUDA(cudaMemcpyAsync(mean, dmean.p, mt * sizeof(double), cudaMemcpyDeviceToHost, s));
      GPGP_CUDA(cudaMemcpyAsync(cov, C.p, (size_t)mt * mt * sizeof(double), cudaMemcpyDeviceToHost, s));
      GPGP_CUDA(cudaStreamSynchronize(s));
      return GPGP_OK;
    }
    cov_matvec(s, m->dk, gm, Ft.p, mt, mt, m->F.p, n, n, m->alpha.p, dmean.p);
    // K(xt, xt), both triangles
    C.alloc(s, (size_t)mt * mt);
    cov_matrix(s, m->dk, gm, Ft.p, mt, mt, Ft.p, mt, mt, C.p, mt, COV_FULL, 1, 1, 0.0, nullptr);
    // aux = L^-1 diag(s) K(x, xt)  (C_chol = diag(sqrt(V)) L)
    R.alloc(s, (size_t)n * mt);
    cov_matrix(s, m->dk, gm, m->F.p, n, n, Ft.p, mt, mt, R.p, n, COV_ROWSCALE, 0, 0, 0.0, m->s.p);
    tmp.alloc(s, (size_t)NB * mt);
    status.alloc(s, 1);
    GPGP_CUDA(cudaMemsetAsync(status.p, 0, sizeof(int), s));
    trsm_lower(s, m->L.p, n, n, m->Winv.p, R.p, mt, n, tmp.p, status.p);
    // cov = K(xt, xt) - aux^T aux + jitter I
    gemm64(s, true, false, mt, mt, n, -1.0, R.p, n, R.p, n, 1.0, C.p, mt);
    add_diag_kernel<<<g1(mt), 256, 0, s>>>(C.p, mt, mt, jitter);
    GPGP_CHECK_LAUNCH();
    GPGP_CUDA(cudaMemcpyAsync(mean, dmean.p, mt * sizeof(double), cudaMemcpyDeviceToHost, s));
    GPGP_CUDA(cudaMemcpyAsync(cov, C.p, (size_t)mt * mt * sizeof(double), cudaMemcpyDeviceToHost, s));
    GPGP_CUDA(cudaStreamSynchronize(s));
    return GPGP_OK;
  });
}

gpgp_status gpgp_mvn_draw(gpgp_ctx *ctx, const double *mean, const double *cov, int64_t d, const double *z,
                          int64_t draws, double *out) {
  if (!ctx || !mean || !cov || !z || !out || d < 1 || draws < 1) return fail(ctx, GPGP_EINVAL, "invalid argument");
  return guarded(ctx, [&]() -> gpgp_status {
    GPGP_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    DBuf dm, C, Z, O, Winv, ldp;
    IBuf status;
    copy_in(s, dm, mean, d, false);
    copy_in(s, C, cov, (size_t)d * d, false);
    copy_in(s, Z, z, (size_t)d * draws, false);
    const int64_t nblk = (d + NB - 1) / NB;
    Winv.alloc(s, (size_t)nblk * NB * NB);
    ldp.alloc(s, nblk + 1);
    status.alloc(s, 1);
    GPGP_CUDA(cudaMemsetAsync(status.p, 0, sizeof(int), s));
    // t(chol(cov)): the lower factor, upper triangle cleared
    potrf(s, C.p, d, d, Winv.p, ldp.p, status.p);
    int hs = 0;
    GPGP_CUDA(cudaMemcpyAsync(&hs, status.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    GPGP_CUDA(cudaStreamSynchronize(s));
    if (hs != 0) return fail(ctx, GPGP_ENOT_PD, "the predictive covariance is not positive definite");
    dim3 g((unsigned)std::min<int64_t>((d + 255) / 256, 64), (unsigned)std::min<int64_t>(d, 65535));
    zero_upper_cols_kernel<<<g, 256, 0, s>>>(C.p, d, d);
    GPGP_CHECK_LAUNCH();
    // out = mean 1^T + L Z
    O.alloc(s, (size_t)d * draws);
    broadcast_cols_kernel<<<(unsigned)std::min<int64_t>((d * draws + 255) / 256, 4096), 256, 0, s>>>(dm.p, d, draws,
                                                                                                    O.p);
    GPGP_CHECK_LAUNCH();
    gemm64(s, false, false, d, draws, d, 1.0, C.p, d, Z.p, d, 1.0, O.p, d);
    GPGP_CUDA(cudaMemcpyAsync(out, O.p, (size_t)d * draws * sizeof(double), cudaMemcpyDeviceToHost, s));
    GPGP_CUDA(cudaStreamSynchronize(s));
    return GPGP_OK;
  });
}

}  // extern "C"
