"""The allocation-free Gaussian fit, checked against the allocating entry point
and the oracle.

gpgp_fit_gaussian_noalloc exists for callers that cannot allocate device
memory when they need a fit (a serving process whose pool already owns all of
HBM, a latency-critical request path, a host framework that forbids
allocation while it drives the GPU). It keeps its scratch in one fixed device
array, so it takes n <= 512. This test calls it through the C ABI on three
problems in a row (the first call on the device is its set-up call) and
compares alpha and the log evidence with gpgp_fit_dev on the same device
inputs and with the oracle, at the FP64 parity tolerance of the other tests
(1e-10 relative). Around each call it reads the device's default memory pool
(the pool the library's stream-ordered allocations come from): its used-memory
high-water mark, reset just before the call, must not rise. From the second
call on, the device's used memory must not rise either: the first use of the
library's code on a device loads the module that holds the fixed array, and
CUDA's lazy module loading makes the array resident then, once. It also checks
that a size beyond the maximum and a NaN input are refused. The file is named
to be collected last.
"""
import copy
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# CUmemPool_attribute values of the CUDA driver API
_POOL_USED_CURRENT = 7
_POOL_USED_HIGH = 8


class _PoolProbe:
    """Device memory in use, read through the driver API: the default memory
    pool's used bytes and high-water mark, and cuMemGetInfo."""

    def __init__(self, device):
        self.cu = C.CDLL("libcuda.so.1")
        self.pool = C.c_void_p()
        assert self.cu.cuDeviceGetDefaultMemPool(C.byref(self.pool), C.c_int(device)) == 0

    def _attr(self, a):
        v = C.c_uint64()
        assert self.cu.cuMemPoolGetAttribute(self.pool, C.c_int(a), C.byref(v)) == 0
        return v.value

    def reset_high(self):
        zero = C.c_uint64(0)  # resets the high-water mark to the current use
        assert self.cu.cuMemPoolSetAttribute(self.pool, C.c_int(_POOL_USED_HIGH), C.byref(zero)) == 0

    def used(self):
        return self._attr(_POOL_USED_CURRENT)

    def high(self):
        return self._attr(_POOL_USED_HIGH)

    def device_used(self):
        free, total = C.c_size_t(), C.c_size_t()
        assert self.cu.cuMemGetInfo_v2(C.byref(free), C.byref(total)) == 0
        return total.value - free.value


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


def test_noalloc_fit_matches_allocating_fit_and_oracle_twice():
    import torch

    import gplite_gb300 as G
    from gplite_gb300 import _lib as L
    from gplite_gb300.gp import kernel_struct
    from oracle import gplite_ref as R

    lib = L.load()
    ctx = L.default_context(0)
    probe = _PoolProbe(0)
    # a larger problem, then a smaller one: a call must not see anything left in
    # the shared scratch by the one before
    cases = [(200, 1, 0.1, [G.cf_sexp(lscale=0.3)]),
             (512, 3, 0.08, [G.cf_sexp(lscale=0.9, magn=1.1), G.cf_const(0.7)]),
             (150, 2, 0.2, [G.cf_matern32(lscale=0.5) * G.cf_lin()])]
    for call, (n, d, sigma, cfs) in enumerate(cases):
        rng = np.random.default_rng(n)
        x = rng.uniform(-2, 2, (n, d))
        y = np.sin(x[:, 0]) + 0.1 * rng.standard_normal(n)
        k = kernel_struct(cfs, d)
        xd = torch.from_numpy(np.ascontiguousarray(x.T)).cuda()  # column-major n x d
        yd = torch.from_numpy(y).cuda()
        ad = torch.zeros(n, dtype=torch.float64, device="cuda")
        lml = np.zeros(1)
        torch.cuda.synchronize()
        used0, dev0 = probe.used(), probe.device_used()
        probe.reset_high()
        st = lib.gpgp_fit_gaussian_noalloc(ctx.h, C.byref(k), sigma, 1e-6, xd.data_ptr(), n, d,
                                           yd.data_ptr(), ad.data_ptr(), L.ptr(lml))
        assert st == 0, L.load().gpgp_last_error(ctx.h)
        torch.cuda.synchronize()
        # nothing was allocated during the call, not even transiently
        assert probe.high() <= used0 and probe.used() == used0
        if call > 0:
            assert probe.device_used() <= dev0
        a_ref, lml_ref = _fit_dev(lib, L, ctx, k, sigma, xd, n, d, yd)
        assert abs(lml[0] - lml_ref) <= 1e-10 * abs(lml_ref)
        alpha = ad.cpu().numpy()
        assert np.allclose(alpha, a_ref, rtol=1e-10, atol=1e-12)
        og = R.gp_init(copy.deepcopy(cfs), R.lik("gaussian", sigma=sigma))
        og = R.gp_fit(og, x, y)
        assert abs(lml[0] - og.fit["log_evidence"]) <= 1e-10 * abs(og.fit["log_evidence"])
        assert np.allclose(alpha, og.fit["alpha"], rtol=1e-9, atol=1e-10)

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
    # a NaN input is refused, and the next call on the same context still works
    n = 40
    x = np.linspace(-1, 1, n)[:, None]
    y = np.sin(3 * x[:, 0])
    y_bad = y.copy()
    y_bad[7] = np.nan
    xd = torch.from_numpy(np.ascontiguousarray(x.T)).cuda()
    ad = torch.zeros(n, dtype=torch.float64, device="cuda")
    st = lib.gpgp_fit_gaussian_noalloc(ctx.h, C.byref(k), 0.3, 1e-6, xd.data_ptr(), n, 1,
                                       torch.from_numpy(y_bad).cuda().data_ptr(), ad.data_ptr(),
                                       L.ptr(lml))
    assert st == L.ENAN and np.isnan(lml[0])
    yd = torch.from_numpy(y).cuda()
    st = lib.gpgp_fit_gaussian_noalloc(ctx.h, C.byref(k), 0.3, 1e-6, xd.data_ptr(), n, 1,
                                       yd.data_ptr(), ad.data_ptr(), L.ptr(lml))
    assert st == 0 and np.isfinite(lml[0])
