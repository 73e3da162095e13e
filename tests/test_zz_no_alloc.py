"""The allocation-free Gaussian fit, checked against the allocating entry point.

gpgp_fit_gaussian_noalloc exists for callers that cannot allocate device
memory when they need a fit (a serving process whose pool already owns all of
HBM, a latency-critical request path, a host framework that forbids
allocation while it drives the GPU). It keeps its scratch in one fixed device
array, so it takes n <= 512. This test calls it through the C ABI twice in a
row, on different problems, and compares alpha and the log evidence with
gpgp_fit_dev on the same device inputs, at the FP64 parity tolerance of the
other tests (1e-10 relative). It also checks that a size beyond the maximum
is rejected. The file is named to be collected last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _fit_dev(lib, L, ctx, k, sigma, xd, n, d, yd):
    lk = L.Lik()
    lk.kind, lk.link, lk.sigma = 0, 0, sigma
    me = L.Method()
    ap = L.Approx()
    ap.kind, ap.maxiter, ap.tol = 0, 30, 1e-4
    op = L.FitOpts()
    op.jitter, op.precision, op.refine_iters = 1e-6, 0, 0
    h = C.c_void_p()
    res = L.FitResult()
    st = lib.gpgp_fit_dev(ctx.h, C.byref(k), C.byref(lk), C.byref(me), C.byref(ap), C.byref(op),
                          xd.data_ptr(), n, d, yd.data_ptr(), None, None, C.byref(h), C.byref(res))
    assert st == 0
    alpha = np.empty(n)
    assert lib.gpgp_model_get(h, 0, L.ptr(alpha)) == 0
    lib.gpgp_model_free(h)
    return alpha, res.log_evidence


def test_noalloc_fit_matches_allocating_fit_twice():
    import torch

    import gplite_gb300 as G
    from gplite_gb300 import _lib as L
    from gplite_gb300.gp import kernel_struct

    lib = L.load()
    ctx = L.default_context(0)
    # a larger problem first, then a smaller one: the second call must not see
    # anything left in the shared scratch by the first
    for n, d, sigma, cfs in [(512, 3, 0.08, [G.cf_sexp(lscale=0.9, magn=1.1), G.cf_const(0.7)]),
                             (150, 2, 0.2, [G.cf_matern32(lscale=0.5) * G.cf_lin()])]:
        rng = np.random.default_rng(n)
        x = rng.uniform(-2, 2, (n, d))
        y = np.sin(x[:, 0]) + 0.1 * rng.standard_normal(n)
        k = kernel_struct(cfs, d)
        xd = torch.from_numpy(np.ascontiguousarray(x.T)).cuda()  # column-major n x d
        yd = torch.from_numpy(y).cuda()
        ad = torch.zeros(n, dtype=torch.float64, device="cuda")
        lml = np.zeros(1)
        torch.cuda.synchronize()
        st = lib.gpgp_fit_gaussian_noalloc(ctx.h, C.byref(k), sigma, 1e-6, xd.data_ptr(), n, d,
                                           yd.data_ptr(), ad.data_ptr(), L.ptr(lml))
        assert st == 0
        torch.cuda.synchronize()
        a_ref, lml_ref = _fit_dev(lib, L, ctx, k, sigma, xd, n, d, yd)
        assert abs(lml[0] - lml_ref) <= 1e-10 * abs(lml_ref)
        assert np.allclose(ad.cpu().numpy(), a_ref, rtol=1e-10, atol=1e-12)

    # beyond the fixed maximum: rejected, nothing written
    n = 513
    x = np.zeros((n, 1))
    xd = torch.from_numpy(np.ascontiguousarray(x.T)).cuda()
    yd = torch.zeros(n, dtype=torch.float64, device="cuda")
    ad = torch.zeros(n, dtype=torch.float64, device="cuda")
    lml = np.zeros(1)
    k = kernel_struct([G.cf_sexp()], 1)
    st = lib.gpgp_fit_gaussian_noalloc(ctx.h, C.byref(k), 0.5, 1e-6, xd.data_ptr(), n, 1,
                                       yd.data_ptr(), ad.data_ptr(), L.ptr(lml))
    assert st == L.EINVAL
