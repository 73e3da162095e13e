// Random-feature methods, method_rf and method_rbf (R/method.R:129-139): the
// reference's feature maps (rf_featmap / rbf_featmap, R/cf.R:532-817) evaluated
// on the device from caller-given draws, the weight-space Laplace iteration
// (laplace_iter.method_rf / laplace.method_rf, R/laplace.R:241-266, 327-355),
// predictions (gp_pred_prior / gp_pred_post.method_rf, R/gp_pred.R:186-200,
// 298-318), the LOO posteriors of a Laplace fit (R/gp_loo.R:119-129) and
// weight-space draws (R/gp_draw.R:87-169). Everything is FP64: the D x D weight
// algebra is small next to the n x D feature matrix, whose Gram matrix is one
// FP64 GEMM.
#include <math.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "model.cuh"

namespace gpgp {

// ---------------------------------------------------------------------------
// feature map
// ---------------------------------------------------------------------------
gpgp_status build_rf_spec(const gpgp_kernel *k, const gpgp_method *me, const DevKernel &dk, RfSpec *sp,
                          std::vector<double> *draws, std::string *err) {
  const bool rbf = me->kind == GPGP_METHOD_RBF;
  sp->nterms = k->nterms;
  sp->ngroups = k->ngroups;
  draws->clear();
  int col = 0;
  for (int g = 0; g < k->ngroups; ++g) {
    sp->gcol0[g] = col;
    int nt = 0, has_cl = 0;
    for (int t = 0; t < k->nterms; ++t)
      if (k->term[t].group == g) {
        ++nt;
        if (k->term[t].kind == GPGP_CF_CONST || k->term[t].kind == GPGP_CF_LIN) has_cl = 1;
      }
    if (nt > 1 && has_cl) {
      *err = rbf ? "RBF features for product kernel containing constant or linear kernel not implemented yet."
                 : "Random features for product kernel containing constant or linear kernel not implemented yet.";
      return GPGP_EUNSUPPORTED;
    }
    const int nb = me->num_basis[g];
    if (nb < 1) {
      *err = "num_basis must be positive";
      return GPGP_EINVAL;
    }
    col += nb;
  }
  sp->gcol0[k->ngroups] = col;
  sp->D = col;
  if (col > 65535) {
    *err = "method_rf / method_rbf: at most 65535 features in total";
    return GPGP_EINVAL;
  }
  for (int t = 0; t < k->nterms; ++t) {
    const gpgp_cf_term &T = k->term[t];
    RfTerm &R = sp->t[t];
    R.group = T.group;
    R.off = dk.t[t].off;
    R.q = dk.t[t].dt;
    R.nb = me->num_basis[T.group];
    R.magn = T.magn;
    R.lscale = T.lscale;
    R.sigma0 = T.sigma0;
    R.sigma = T.sigma;
    R.doff = (int64_t)draws->size();
    int64_t nd = 0;
    switch (T.kind) {
      case GPGP_CF_CONST:
      case GPGP_CF_LIN:
        if (T.periodic) {
          *err = "random features of cf_periodic around cf_const or cf_lin are not supported";
          return GPGP_EUNSUPPORTED;
        }
        R.kind = T.kind == GPGP_CF_CONST ? RF_CONST : RF_LIN;
        if (R.nb != (T.kind == GPGP_CF_CONST ? 1 : R.q)) {
          *err = "num_basis of cf_const must be 1 and of cf_lin its number of inputs (check_num_basis)";
          return GPGP_EINVAL;
        }
        break;
      case GPGP_CF_SEXP:
        if (rbf) {
          R.kind = RBF_SEXP;
          nd = (int64_t)R.q * R.nb;
        } else {
          if (R.nb % 2 == 1) {
            *err = "number of features must be an even number.";
            return GPGP_EINVAL;
          }
          R.kind = RF_SEXP;
          nd = (int64_t)R.q * (R.nb / 2);
        }
        break;
      case GPGP_CF_NN:
        if (rbf) {
          *err = "RBF features are not available for cf_nn";
          return GPGP_EUNSUPPORTED;
        }
        R.kind = RF_NN;
        nd = (int64_t)R.q * R.nb + R.nb;
        break;
      default:
        *err = rbf ? "RBF features are not available for Matern kernels"
                   : "Random Fourier features for Matern kernels not implemented yet.";
        return GPGP_EUNSUPPORTED;
    }
    if (nd > 0) {
      if (!me->draws[t]) {
        *err = "method_rf / method_rbf: the draws of a term are missing";
        return GPGP_EINVAL;
      }
      draws->insert(draws->end(), me->draws[t], me->draws[t] + nd);
    }
  }
  return GPGP_OK;
}

// One term's feature j at one point; x points at the point's first input of the
// term, consecutive inputs ldf apart.
__device__ __forceinline__ double rf_term_value(const RfTerm &T, const double *x, int64_t ldf,
                                                const double *__restrict__ dr, int j) {
  switch (T.kind) {
    case RF_CONST:
      return T.magn;  // magn * rep(1, n) (R/cf.R:553-559)
    case RF_LIN:
      return T.magn * x[j * ldf];  // magn * x (R/cf.R:561-569)
    case RF_SEXP: {
      // h = x w, w = rnorm(q m) / lscale; magn sqrt(1/m) [cos(h), sin(h)] (R/cf.R:571-610)
      const int m = T.nb / 2;
      const int jj = j < m ? j : j - m;
      const double sc = 1.0 / T.lscale;
      const double *w = dr + T.doff + (int64_t)jj * T.q;
      double h = 0.0;
      for (int c = 0; c < T.q; ++c) h = fma(x[c * ldf], w[c] * sc, h);
      const double a = T.magn * sqrt(1.0 / m);
      return j < m ? a * cos(h) : a * sin(h);
    }
    case RF_NN: {
      // erf(w0 + x w), w = rnorm(q m) sigma, w0 = rnorm(m) sigma0 sigma; magn / sqrt(m) (R/cf.R:622-657)
      const int m = T.nb;
      const double *w = dr + T.doff + (int64_t)j * T.q;
      double h = dr[T.doff + (int64_t)T.q * m + j] * T.sigma0 * T.sigma;
      for (int c = 0; c < T.q; ++c) h = fma(x[c * ldf], w[c] * T.sigma, h);
      return (T.magn / sqrt((double)m)) * erf(h);
    }
    default: {
      // exp(-|x - centre_j|^2 / lscale^2) magn sqrt(1/nb) (R/cf.R:740-775)
      const double *cj = dr + T.doff + (int64_t)j * T.q;
      double r2 = 0.0;
      for (int c = 0; c < T.q; ++c) {
        const double d = x[c * ldf] - cj[c];
        r2 += d * d;
      }
      return (T.magn * sqrt(1.0 / T.nb)) * exp(-r2 / (T.lscale * T.lscale));
    }
  }
}

// Z (n x D, ldz): column c belongs to group g; a group's features are the
// products of its terms' features (cf_prod, R/cf.R:676-695). Columns of groups
// outside gmask are zero. One column per grid row, points along x (coalesced).
__global__ void rf_features_kernel(RfSpec sp, uint32_t gmask, const double *__restrict__ F, int64_t ldf,
                                   int64_t n, const double *__restrict__ dr, double *__restrict__ Z,
                                   int64_t ldz) {
  const int c = blockIdx.y;
  int g = 0;
  while (g + 1 < sp.ngroups && c >= sp.gcol0[g + 1]) ++g;
  const int j = c - sp.gcol0[g];
  const bool on = (gmask >> g) & 1u;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double z = 0.0;
    if (on) {
      z = 1.0;
      for (int t = 0; t < sp.nterms; ++t)
        if (sp.t[t].group == g) z *= rf_term_value(sp.t[t], F + i + sp.t[t].off * ldf, ldf, dr, j);
    }
    Z[i + c * ldz] = z;
  }
}

static void rf_features(cudaStream_t s, const RfSpec &sp, uint32_t gmask, const double *F, int64_t ldf,
                        int64_t n, const double *dr, double *Z, int64_t ldz) {
  if (n == 0 || sp.D == 0) return;
  dim3 grid((unsigned)std::min<int64_t>((n + 255) / 256, 1024), (unsigned)sp.D);
  rf_features_kernel<<<grid, 256, 0, s>>>(sp, gmask, F, ldf, n, dr, Z, ldz);
  GPGP_CHECK_LAUNCH();
}

// ---------------------------------------------------------------------------
// small kernels
// ---------------------------------------------------------------------------
// Zv = Z / V (rows), r = z / V; flags |= 2 on NaN in V or z
__global__ void rf_scale_kernel(int64_t n, int64_t D, const double *__restrict__ Z, const double *__restrict__ V,
                                const double *__restrict__ z, double *__restrict__ Zv, double *__restrict__ r,
                                int *flags) {
  const int64_t tot = n * D;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < tot; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e % n;
    Zv[e] = Z[e] / V[i];
    if (e < n) {
      r[e] = z[e] / V[e];
      if (V[e] != V[e] || z[e] != z[e]) atomicOr(flags, 2);
    }
  }
}

__global__ void rf_add_identity_kernel(double *H, int64_t D) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < D) H[i + i * D] += 1.0;
}

__global__ void rf_zero_upper_kernel(double *A, int64_t D) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e < D * D) {
    const int64_t i = e % D, j = e / D;
    if (i < j) A[e] = 0.0;
  }
}

// out (rows x cols) = A[idx, idx] (A ld lda) and v_out = v[idx]
__global__ void rf_gather_kernel(const double *__restrict__ A, int64_t lda, const double *__restrict__ v,
                                 const int *__restrict__ idx, int64_t k, double *__restrict__ out,
                                 double *__restrict__ vout) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e < k * k) {
    const int64_t i = e % k, j = e / k;
    out[e] = A[idx[i] + (int64_t)idx[j] * lda];
  }
  if (e < k) vout[e] = v[idx[e]];
}

// Wd (D x draws) = 0; rows idx[i] <- mean_i + (Lz)_i,
__global__ void rf_scatter_kernel(const double *__restrict__ W, const double *__restrict__ mean,
                                  const int *__restrict__ idx, int64_t k, int64_t D, int64_t draws,
                                  double *__restrict__ Wd) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e < k * draws) {
    const int64_t i = e % k, c = e / k;
    Wd[idx[i] + c * D] = mean[i] + W[e];
  }
}

__global__ void rf_row_sumsq_kernel(const double *__restrict__ Z, int64_t n, int64_t D, double *__restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = 0.0;
  for (int64_t c = 0; c < D; ++c) {
    const double v = Z[i + c * n];
    s += v * v;
  }
  out[i] = s;
}

// ---------------------------------------------------------------------------
// fit: laplace.method_rf (R/laplace.R:327-351) over laplace_iter.method_rf
// (R/laplace.R:241-262)
// ---------------------------------------------------------------------------
gpgp_status fit_rf(gpgp_model *m, gpgp_fit_result *res) {
  gpgp_ctx *ctx = m->ctx;
  cudaStream_t st = ctx->stream;
  const int64_t n = m->n;
  if (m->approx.kind != GPGP_APPROX_LAPLACE)
    return fail(ctx, GPGP_EUNSUPPORTED,
                "approx_ep is not available for method_rf / method_rbf (the reference has no EP for them)");
  RfState &R = *m->rf;
  const int64_t D = R.spec.D;
  R.Z.alloc(st, (size_t)n * D);
  rf_features(st, R.spec, 0xffffffffu, m->F.p, n, n, R.dr.p, R.Z.p, n);
  const double *trials = m->has_trials ? m->trials.p : nullptr;
  const double *offset = m->has_offset ? m->offset.p : nullptr;
  const int64_t nblk = (D + NB - 1) / NB;
  DBuf Zv, rhs, b, t1, what, fnew, red, lp;
  IBuf status, flags;
  Zv.alloc(st, (size_t)n * D);
  rhs.alloc(st, n);
  b.alloc(st, D);
  t1.alloc(st, D);
  what.alloc(st, D);
  fnew.alloc(st, n);
  red.alloc(st, 256);
  lp.alloc(st, nblk + 1);
  status.alloc(st, 1);
  flags.alloc(st, 1);
  R.L.alloc(st, (size_t)D * D);
  R.Wblk.alloc(st, (size_t)nblk * NB * NB);
  m->fmean.alloc(st, n);
  m->z.alloc(st, n);
  m->V.alloc(st, n);
  GPGP_CUDA(cudaMemsetAsync(m->fmean.p, 0, n * sizeof(double), st));
  const int maxiter = m->lik.kind == GPGP_LIK_GAUSSIAN ? 1 : std::max(1, m->approx.maxiter);
  double diff = 0.0;
  int it;
  res->iters = 0;
  res->converged = 1;
  res->quad_ok = 1;
  res->info = 0;
  const unsigned gz = (unsigned)std::min<int64_t>(((int64_t)n * D + 255) / 256, 8192);
  for (it = 1; it <= maxiter; ++it) {
    lik_pseudodata_la(st, m->lk, n, m->fmean.p, m->y.p, trials, offset, m->z.p, m->V.p);
    GPGP_CUDA(cudaMemsetAsync(flags.p, 0, sizeof(int), st));
    GPGP_CUDA(cudaMemsetAsync(status.p, 0, sizeof(int), st));
    rf_scale_kernel<<<gz, 256, 0, st>>>(n, D, R.Z.p, m->V.p, m->z.p, Zv.p, rhs.p, flags.p);
    GPGP_CHECK_LAUNCH();
    // H = t(Z) %*% (Z / V) + I, L = t(chol(H + I))
    gemm64(st, true, false, D, D, n, 1.0, R.Z.p, n, Zv.p, n, 0.0, R.L.p, D);
    rf_add_identity_kernel<<<g1(D), 256, 0, st>>>(R.L.p, D);
    GPGP_CHECK_LAUNCH();
    potrf(st, R.L.p, D, D, R.Wblk.p, lp.p, status.p);
    // what = backsolve(t(L), forwardsolve(L, t(Z) %*% (z / V)))
    gemv64(st, true, n, D, 1.0, R.Z.p, n, rhs.p, 0.0, b.p);
    trsv_lower(st, R.L.p, D, D, R.Wblk.p, b.p, t1.p, status.p);
    trsv_lower_t(st, R.L.p, D, D, R.Wblk.p, t1.p, what.p, status.p);
    gemv64(st, false, n, D, 1.0, R.Z.p, n, what.p, 0.0, fnew.p);  // fhat_new = Z %*% what
    int hs[2] = {0, 0};
    GPGP_CUDA(cudaMemcpyAsync(&hs[0], status.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    GPGP_CUDA(cudaMemcpyAsync(&hs[1], flags.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    GPGP_CUDA(cudaStreamSynchronize(st));
    if (hs[1] & 2) {
      res->status = GPGP_ENAN;
      res->log_evidence = NAN;
      return fail(ctx, GPGP_ENAN, "NaN in the Laplace pseudo-data");
    }
    if (hs[0] != 0) {
      res->status = GPGP_ENOT_PD;
      res->info = hs[0];
      res->log_evidence = -INFINITY;
      return fail(ctx, GPGP_ENOT_PD, "chol(H + I) failed: the weight posterior precision is not positive definite");
    }
    max_abs_diff(st, n, m->fmean.p, fnew.p, red.p);
    diff = read_scalar(ctx, red.p + 64);
    GPGP_CUDA(cudaMemcpyAsync(m->fmean.p, fnew.p, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
    if (diff < m->approx.tol) break;
  }
  if (it > maxiter) it = maxiter;
  res->iters = it;
  if (maxiter > 1 && it == maxiter && !(diff < m->approx.tol)) res->converged = 0;
  // log_evidence = n/2 log(2 pi) + wcov_logdet / 2 + log_prior + log_lik (R/laplace.R:256-259)
  lik_loglik(st, m->lk, n, m->fmean.p, m->y.p, trials, offset, red.p + 101, red.p);
  dot_partial(st, D, what.p, what.p, red.p + 110);  // at red + 174
  sum_vec(st, lp.p, nblk, red.p + 102);
  const double ll = read_scalar(ctx, red.p + 101);
  const double ww = read_scalar(ctx, red.p + 174);
  const double ldL = read_scalar(ctx, red.p + 102);
  const double two_pi = 2.0 * 3.14159265358979323846;
  const double wcov_logdet = -2.0 * ldL;
  const double log_prior = -0.5 * (double)D * log(two_pi) - 0.5 * ww;
  m->log_evidence = 0.5 * (double)n * log(two_pi) + 0.5 * wcov_logdet + log_prior + ll;
  // weight posterior: wmean = what, W = L^-1, wcov = W^T W
  R.wmean.alloc(st, D);
  GPGP_CUDA(cudaMemcpyAsync(R.wmean.p, what.p, D * sizeof(double), cudaMemcpyDeviceToDevice, st));
  R.W.alloc(st, (size_t)D * D);
  {
    DBuf tmp;
    tmp.alloc(st, (size_t)NB * D);
    trtri_lower(st, R.L.p, D, D, R.Wblk.p, R.W.p, D, tmp.p, status.p);
  }
  R.wcov.alloc(st, (size_t)D * D);
  gemm64(st, true, false, D, D, D, 1.0, R.W.p, D, R.W.p, D, 0.0, R.wcov.p, D);
  res->log_evidence = m->log_evidence;
  res->status = GPGP_OK;
  return GPGP_OK;
}

// mean = zt wmean, var = diag(zt wcov zt^T) = |W zt_i|^2 (zt: columns outside gm zero)
gpgp_status pred_rf(gpgp_model *m, const double *Ft, int64_t mt, uint32_t gm, double *mean, double *var) {
  cudaStream_t st = m->ctx->stream;
  RfState &R = *m->rf;
  const int64_t D = R.spec.D;
  if (mt == 0) return GPGP_OK;
  DBuf Zt;
  Zt.alloc(st, (size_t)mt * D);
  rf_features(st, R.spec, gm, Ft, mt, mt, R.dr.p, Zt.p, mt);
  gemv64(st, false, mt, D, 1.0, Zt.p, mt, R.wmean.p, 0.0, mean);
  if (var) {
    DBuf T;
    T.alloc(st, (size_t)D * mt);
    gemm64(st, false, true, D, mt, D, 1.0, R.W.p, D, Zt.p, mt, 0.0, T.p, D);
    col_sumsq(st, T.p, D, mt, D, var);
  }
  return GPGP_OK;
}

// posterior variances at the training inputs (gp_pred_post(train = TRUE), R/gp_loo.R:124)
void rf_train_var(gpgp_model *m, double *var) {
  cudaStream_t st = m->ctx->stream;
  RfState &R = *m->rf;
  const int64_t D = R.spec.D, n = m->n;
  DBuf T;
  T.alloc(st, (size_t)D * n);
  gemm64(st, false, true, D, n, D, 1.0, R.W.p, D, R.Z.p, n, 0.0, T.p, D);
  col_sumsq(st, T.p, D, n, D, var);
}

// the columns of the groups in gm
static std::vector<int> rf_selected(const RfSpec &sp, uint32_t gm) {
  std::vector<int> idx;
  for (int g = 0; g < sp.ngroups; ++g)
    if ((gm >> g) & 1u)
      for (int c = sp.gcol0[g]; c < sp.gcol0[g + 1]; ++c) idx.push_back(c);
  return idx;
}

}  // namespace gpgp

using namespace gpgp;

extern "C" {

gpgp_status gpgp_rf_prior(gpgp_ctx *ctx, const gpgp_kernel *k, const gpgp_method *method, const double *xt,
                          int64_t m, int32_t d, uint32_t group_mask, double *var, const double *z, int64_t draws,
                          double *sample) {
  if (!ctx || !k || !method || !xt || m < 0 || d < 1 || (z && (!sample || draws < 1)))
    return fail(ctx, GPGP_EINVAL, "invalid argument");
  if (method->kind != GPGP_METHOD_RF && method->kind != GPGP_METHOD_RBF)
    return fail(ctx, GPGP_EINVAL, "gpgp_rf_prior needs method_rf or method_rbf");
  return guarded(ctx, [&]() -> gpgp_status {
    GPGP_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    DevKernel dk;
    std::vector<HostTermPrep> prep;
    std::string err;
    gpgp_status s0 = build_dev_kernel(k, d, &dk, &prep, &err);
    if (s0 != GPGP_OK) return fail(ctx, s0, err);
    RfSpec sp;
    std::vector<double> hd;
    s0 = build_rf_spec(k, method, dk, &sp, &hd, &err);
    if (s0 != GPGP_OK) return fail(ctx, s0, err);
    const uint32_t gm = group_mask ? group_mask : 0xffffffffu;
    const std::vector<int> sel = rf_selected(sp, gm);
    const int64_t D = sp.D, ks = (int64_t)sel.size();
    if (m == 0) return GPGP_OK;
    DBuf x, F, dr, Zt;
    copy_in(st, x, xt, (size_t)m * d, false);
    F.alloc(st, (size_t)m * std::max(1, dk.nfeat));
    prep_features(st, dk, prep, x.p, m, m, F.p, m);
    dr.alloc(st, std::max<size_t>(1, hd.size()));
    if (!hd.empty())
      GPGP_CUDA(cudaMemcpyAsync(dr.p, hd.data(), hd.size() * sizeof(double), cudaMemcpyHostToDevice, st));
    Zt.alloc(st, (size_t)m * D);
    rf_features(st, sp, gm, F.p, m, m, dr.p, Zt.p, m);
    if (var) {
      // diag(zt %*% t(zt)) (R/gp_pred.R:195-197)
      DBuf v;
      v.alloc(st, m);
      rf_row_sumsq_kernel<<<g1(m), 256, 0, st>>>(Zt.p, m, D, v.p);
      GPGP_CHECK_LAUNCH();
      GPGP_CUDA(cudaMemcpyAsync(var, v.p, m * sizeof(double), cudaMemcpyDeviceToHost, st));
      GPGP_CUDA(cudaStreamSynchronize(st));
    }
    if (z) {
      // zt %*% w, w ~ N(0, I) over the selected features (R/gp_draw.R:93-96)
      DBuf zd, Wd, out;
      IBuf idx;
      copy_in(st, zd, z, (size_t)ks * draws, false);
      idx.alloc(st, std::max<int64_t>(1, ks));
      if (ks) GPGP_CUDA(cudaMemcpyAsync(idx.p, sel.data(), ks * sizeof(int), cudaMemcpyHostToDevice, st));
      DBuf zero;
      zero.alloc(st, std::max<int64_t>(1, ks));
      GPGP_CUDA(cudaMemsetAsync(zero.p, 0, std::max<int64_t>(1, ks) * sizeof(double), st));
      Wd.alloc(st, (size_t)D * draws);
      GPGP_CUDA(cudaMemsetAsync(Wd.p, 0, (size_t)D * draws * sizeof(double), st));
      if (ks) {
        rf_scatter_kernel<<<g1(ks * draws), 256, 0, st>>>(zd.p, zero.p, idx.p, ks, D, draws, Wd.p);
        GPGP_CHECK_LAUNCH();
      }
      out.alloc(st, (size_t)m * draws);
      gemm64(st, false, false, m, draws, D, 1.0, Zt.p, m, Wd.p, D, 0.0, out.p, m);
      GPGP_CUDA(cudaMemcpyAsync(sample, out.p, (size_t)m * draws * sizeof(double), cudaMemcpyDeviceToHost, st));
      GPGP_CUDA(cudaStreamSynchronize(st));
    }
    return GPGP_OK;
  });
}

gpgp_status gpgp_rf_draw(gpgp_model *model, const double *xt, int64_t m, uint32_t group_mask, const double *z,
                         int64_t draws, double *sample) {
  if (!model || !xt || !z || !sample || m < 0 || draws < 1)
    return fail(model ? model->ctx : nullptr, GPGP_EINVAL, "invalid argument");
  if (!model->rf) return fail(model->ctx, GPGP_EINVAL, "gpgp_rf_draw needs a method_rf / method_rbf model");
  if (!model->fitted) return fail(model->ctx, GPGP_ENOT_FITTED, "model is not fitted");
  gpgp_ctx *ctx = model->ctx;
  return guarded(ctx, [&]() -> gpgp_status {
    GPGP_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    RfState &R = *model->rf;
    const uint32_t gm = group_mask ? group_mask : 0xffffffffu;
    const std::vector<int> sel = rf_selected(R.spec, gm);
    const int64_t D = R.spec.D, ks = (int64_t)sel.size(), d = model->d;
    if (m == 0) return GPGP_OK;
    if (ks == 0) return fail(ctx, GPGP_EINVAL, "no covariance function selected");
    DBuf x, F, Zt, C, wm, zd, T, Wd, out, lp;
    IBuf idx, status;
    copy_in(st, x, xt, (size_t)m * d, false);
    F.alloc(st, (size_t)m * std::max(1, model->dk.nfeat));
    prep_features(st, model->dk, model->prep, x.p, m, m, F.p, m);
    Zt.alloc(st, (size_t)m * D);
    rf_features(st, R.spec, gm, F.p, m, m, R.dr.p, Zt.p, m);
    // chol of the selected block of wcov (get_w_cov, R/gp.R:256-262)
    idx.alloc(st, ks);
    GPGP_CUDA(cudaMemcpyAsync(idx.p, sel.data(), ks * sizeof(int), cudaMemcpyHostToDevice, st));
    C.alloc(st, (size_t)ks * ks);
    wm.alloc(st, ks);
    rf_gather_kernel<<<g1(ks * ks), 256, 0, st>>>(R.wcov.p, D, R.wmean.p, idx.p, ks, C.p, wm.p);
    GPGP_CHECK_LAUNCH();
    const int64_t nblk = (ks + NB - 1) / NB;
    DBuf Wb;
    Wb.alloc(st, (size_t)nblk * NB * NB);
    lp.alloc(st, nblk + 1);
    status.alloc(st, 1);
    GPGP_CUDA(cudaMemsetAsync(status.p, 0, sizeof(int), st));
    potrf(st, C.p, ks, ks, Wb.p, lp.p, status.p);
    rf_zero_upper_kernel<<<g1(ks * ks), 256, 0, st>>>(C.p, ks);
    GPGP_CHECK_LAUNCH();
    int hs = 0;
    GPGP_CUDA(cudaMemcpyAsync(&hs, status.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    GPGP_CUDA(cudaStreamSynchronize(st));
    if (hs != 0) return fail(ctx, GPGP_ENOT_PD, "chol(wcov) failed");
    // w = wmean + t(chol(wcov)) z (mvnrnd, R/gp_draw.R:182-188); sample = zt w
    copy_in(st, zd, z, (size_t)ks * draws, false);
    T.alloc(st, (size_t)ks * draws);
    gemm64(st, false, false, ks, draws, ks, 1.0, C.p, ks, zd.p, ks, 0.0, T.p, ks);
    Wd.alloc(st, (size_t)D * draws);
    GPGP_CUDA(cudaMemsetAsync(Wd.p, 0, (size_t)D * draws * sizeof(double), st));
    rf_scatter_kernel<<<g1(ks * draws), 256, 0, st>>>(T.p, wm.p, idx.p, ks, D, draws, Wd.p);
    GPGP_CHECK_LAUNCH();
    out.alloc(st, (size_t)m * draws);
    gemm64(st, false, false, m, draws, D, 1.0, Zt.p, m, Wd.p, D, 0.0, out.p, m);
    GPGP_CUDA(cudaMemcpyAsync(sample, out.p, (size_t)m * draws * sizeof(double), cudaMemcpyDeviceToHost, st));
    GPGP_CUDA(cudaStreamSynchronize(st));
    return GPGP_OK;
  });
}

}  // extern "C"
