"""Mixed-precision path (BF16-sliced tcgen05 products, FP64 diagonal blocks,
FP64 log-determinant, FP64 iterative refinement) against the oracle.

Tolerances, written here as the contract: log evidence 1e-8 relative (the
stated bar for the mixed path); posterior mean and alpha 1e-9 of the largest
entry; posterior variance 1e-6 relative per entry; gradient 1e-8 of the
largest entry; LOO densities 1e-7 of the largest entry.
"""
import ctypes as C
import warnings

import numpy as np
import pytest

import gplite_gb300 as G
from gplite_gb300 import _lib as L
from oracle import gplite_ref as R
from helpers import oracle_gp

pytestmark = pytest.mark.gpu


def relmax(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / np.max(np.abs(np.asarray(b))))


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300)))


# 4 slices keep 32 bits of each row (truncation 2^-33 of the row maximum),
# 5 slices 40 bits (2^-41): the bounds leave a factor ~10 over those figures
# for the random operands, whose entries spread over 2^8 in magnitude.
@pytest.mark.parametrize("slices,bound", [(4, 2e-9), (5, 1e-11)])
@pytest.mark.parametrize("M,N,K", [(128, 64, 64), (300, 200, 130), (1000, 500, 640), (64, 700, 1),
                                   (96, 40, 300)])
def test_sliced_gemm_selftest(M, N, K, slices, bound):
    ctx = L.default_context(0)
    e = C.c_double(-1.0)
    st = L.load().gpgp_mixed_selftest(ctx.h, M, N, K, slices, C.byref(e))
    assert st == 0
    assert 0 <= e.value < bound, e.value


@pytest.mark.parametrize("kind", ["sexp", "matern32", "matern52_const", "prod_sum"])
def test_double_float_covariance_matches_fp64(kind):
    """Under mixed precision K and its derivative matrices are evaluated in
    double-float arithmetic (gpgp_cov_df_selftest against the FP64 kernels):
    max-norm relative difference <= 1e-13 over K and every derivative matrix;
    per entry of K (entries above 1e-20 of the largest) <= 1e-11: the relative
    error of e^-a grows with a (~a 2^-44). Derivative entries proportional to
    the squared distance are held in the max norm only: near-coincident points
    amplify the inputs' 48-bit representation error relative to that distance."""
    from gplite_gb300 import gp as GP
    rng = np.random.default_rng(3)
    n, d = 700, 3
    x = rng.uniform(-1, 1, (n, d)) * np.array([1.0, 2.0, 0.5])
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")  # a product with two free magnitudes warns (R/misc.R:76)
        cfs = {"sexp": [G.cf_sexp(lscale=0.4, magn=1.3)], "matern32": [G.cf_matern32(lscale=0.7)],
               "matern52_const": [G.cf_matern52(lscale=0.6), G.cf_const(0.8)],
               "prod_sum": [G.cf_const(0.9) * G.cf_matern52(lscale=0.5, vars=[0, 1]),
                            G.cf_sexp(lscale=0.3, vars=[2])]}[kind]
    k = GP.kernel_struct(cfs, d)
    err = (C.c_double * 2)()
    xf = L.fortran(x)
    ctx = L.default_context()
    st = L.load().gpgp_cov_df_selftest(ctx.h, C.byref(k), L.ptr(xf), n, d, 1e-6, err)
    L.check(st, ctx.h)
    assert err[0] <= 1e-13 and err[1] <= 1e-11, (kind, err[0], err[1])


@pytest.mark.parametrize("n", [65, 200, 700, 2048])
def test_mixed_gaussian_matches_oracle(n):
    rng = np.random.default_rng(n)
    x = rng.uniform(-1, 1, (n, 8))
    xt = rng.uniform(-1, 1, (257, 8))
    y = np.sin(2 * x[:, 0]) + x[:, 1] + 0.05 * rng.standard_normal(n)

    def mk():
        return G.gp_init([G.cf_matern52(lscale=0.7), G.cf_const(1.0)], G.lik_gaussian(sigma=0.05))

    gm = G.gp_fit(mk(), x, y, precision="mixed")
    g6 = G.gp_fit(mk(), x, y)
    og = R.gp_fit(oracle_gp(mk()), x, y)
    assert rel(gm.fit["log_evidence"], og.fit["log_evidence"]) < 1e-8
    assert relmax(G.model_field(gm, "alpha"), og.fit["alpha"]) < 1e-9
    pm, po = G.gp_pred(gm, xt, var=True), R.gp_pred(og, xt, var=True)
    assert relmax(pm["mean"], po["mean"]) < 1e-9
    assert rel(pm["var"], po["var"]) < 1e-6
    assert relmax(G.gp_energy_grad(gm), G.gp_energy_grad(g6)) < 1e-8
    assert relmax(G.gp_loo(gm, x, y)["loos"], R.gp_loo(og, x, y)["loos"]) < 1e-7


@pytest.mark.parametrize("approx", ["laplace", "ep"])
def test_mixed_bernoulli_matches_oracle(approx):
    rng = np.random.default_rng(3)
    n = 700
    x = rng.standard_normal((n, 4))
    f = 2 * np.sin(x[:, 0])
    y = (rng.uniform(size=n) < 1 / (1 + np.exp(-f))).astype(float)
    ap = G.approx_laplace(tol=1e-6) if approx == "laplace" else G.approx_ep()

    def mk():
        return G.gp_init(G.cf_sexp(lscale=0.5, magn=2.0), G.lik_bernoulli(), approx=ap)

    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        gm = G.gp_fit(mk(), x, y, precision="mixed")
        og = R.gp_fit(oracle_gp(mk()), x, y)
    assert gm.fit["iters"] == og.fit["iters"]
    assert rel(gm.fit["log_evidence"], og.fit["log_evidence"]) < 1e-8
    assert relmax(G.gp_loo(gm, x, y)["loos"], R.gp_loo(og, x, y)["loos"]) < 1e-7


def _poisson_counts(scale, seed, n=300):
    rng = np.random.default_rng(seed)
    x = rng.uniform(-2, 2, (n, 2))
    w = rng.standard_normal((2, 64)) / 0.37
    b = rng.uniform(0, 2 * np.pi, 64)
    f = np.sqrt(2.0 / 64) * (np.cos(x @ w + b) @ rng.standard_normal(64))
    return x, rng.poisson(np.exp(scale * f)).astype(float)


def test_mixed_laplace_never_fails_where_fp64_does_not():
    """Poisson data with large counts on which the reference's Laplace iteration
    oscillates (the oracle reaches its 30-iteration limit on these seeds, and some
    trajectories overflow into the non-log-concave branch): a mixed fit that breaks
    down is redone in FP64 and then equals the plain result exactly; a mixed fit
    never raises where the plain one does not; converged plain fits are matched
    within 1e-8 of max(|LML|, n)."""
    import warnings
    compared = 0
    for scale, seed in [(1.3, 1), (1.3, 2), (1.2, 6), (1.3, 6), (1.3, 11), (1.0, 0), (1.0, 3)]:
        x, y = _poisson_counts(scale, seed)
        out = {}
        for prec in ("fp64", "mixed"):
            gp = G.gp_init(G.cf_sexp(lscale=0.37, magn=1.0), G.lik_poisson())
            with warnings.catch_warnings():
                warnings.simplefilter("ignore")
                try:
                    gp = G.gp_fit(gp, x, y, precision=prec)
                    out[prec] = gp.fit
                except L.GpgpError as e:
                    out[prec] = e.status
        f, m = out["fp64"], out["mixed"]
        if not isinstance(f, dict):
            assert not isinstance(m, dict) and m == f
            continue
        assert isinstance(m, dict), (scale, seed, m)
        if m["precision_used"] == "fp64":
            assert m["log_evidence"] == f["log_evidence"]
        elif f["converged"] and m["converged"]:
            assert abs(m["log_evidence"] - f["log_evidence"]) <= 1e-8 * max(abs(f["log_evidence"]), len(y))
            compared += 1
    assert compared >= 1


@pytest.mark.parametrize("n", [700, 1214, 2248])
def test_mixed_gradient_and_inverse_match_fp64(n):
    """The energy gradient needs B^-1 = W^T W with W = L^-1 (the triangular inverse
    assembled from batched 128/256/512 diagonal levels plus a recursion above them;
    sizes that are not powers of two exercise the remainder blocks): the mixed
    gradient and predictive variances agree with the FP64 path."""
    rng = np.random.default_rng(n)
    x = rng.uniform(-1, 1, (n, 3))
    y = np.sin(3 * x[:, 0]) + x[:, 1] + 0.05 * rng.standard_normal(n)
    xt = rng.uniform(-1, 1, (97, 3))
    out = {}
    for prec in ("fp64", "mixed"):
        gp = G.gp_init([G.cf_matern52(lscale=0.6, magn=1.0), G.cf_const(magn=0.7)], G.lik_gaussian(sigma=0.05))
        gp = G.gp_fit(gp, x, y, precision=prec)
        out[prec] = (G.gp_energy_grad(gp), G.gp_pred(gp, xt, var=True))
    g64, p64 = out["fp64"]
    gm, pm = out["mixed"]
    assert relmax(gm, g64) < 1e-7
    # var = k(x, x) - |L^-1 k|^2 cancels (here 1.49 - 1.49 -> 1e-3): the sliced products of
    # the triangular inverse carry ~2^-33 of their operands per level, which accumulates to
    # ~1.5e-8 of the prior variance at n ~ 1000-2000 (measured), so the bound is on that scale
    prior_var = 1.0 ** 2 + 0.7 ** 2
    assert np.max(np.abs(pm["var"] - p64["var"])) < 1e-7 * prior_var
    assert relmax(pm["mean"], p64["mean"]) < 1e-8


def _fit_grad_abi(gp, x, y, prec, fused):
    """gpgp_fit_grad, or gpgp_fit then gpgp_model_grad, through the C ABI."""
    from gplite_gb300 import gp as GP
    lib = L.load()
    ctx = L.default_context()
    n, d = x.shape
    GP.learn_scales(gp, x)
    k = GP.kernel_struct(gp.cfs, d)
    lk = GP._lik_struct(gp.lik)
    me, keep = GP._method_struct(gp, d, x)
    ap = GP._approx_struct(gp)
    op = L.FitOpts()
    op.jitter, op.precision, op.refine_iters = 1e-6, L.PRECISION[prec], 2
    xf, yy = L.fortran(x), np.ascontiguousarray(y)
    h = C.c_void_p()
    res = L.FitResult()
    gt = np.zeros(len(GP._flat_terms(gp)) * L.TERM_NPARAM)
    gs = C.c_double(0.0)
    if fused:
        st = lib.gpgp_fit_grad(ctx.h, C.byref(k), C.byref(lk), C.byref(me), C.byref(ap), C.byref(op), L.ptr(xf),
                               n, d, L.ptr(yy), None, None, C.byref(h), C.byref(res), L.ptr(gt), C.byref(gs))
        L.check(st, ctx.h)
    else:
        L.check(lib.gpgp_fit(ctx.h, C.byref(k), C.byref(lk), C.byref(me), C.byref(ap), C.byref(op), L.ptr(xf),
                             n, d, L.ptr(yy), None, None, C.byref(h), C.byref(res)), ctx.h)
        L.check(lib.gpgp_model_grad(h, L.ptr(gt), C.byref(gs)), ctx.h)
    lib.gpgp_model_free(h)
    return res.log_evidence, np.append(gt, gs.value)


@pytest.mark.parametrize("n", [700, 2248])
def test_fit_grad_entry_point(n):
    """gpgp_fit_grad = gpgp_fit + gpgp_model_grad. In FP64 the two factor the same K;
    at n = 2248 the fused call's gradient is a pass over K's derivative matrices
    written with K (summed in another order than the separate call's regenerated
    tiles: 1e-12). Under mixed precision the fused call also solves for alpha with
    W = L^-1 (formed right after the factor) and its results agree with the separate
    calls (1e-10 on the evidence) and with FP64 within the mixed path's bound (1e-8)."""
    rng = np.random.default_rng(n + 1)
    x = rng.uniform(-1, 1, (n, 3))
    y = np.sin(3 * x[:, 0]) + x[:, 1] + 0.05 * rng.standard_normal(n)

    def gp():
        return G.gp_init([G.cf_matern52(lscale=0.6, magn=1.0), G.cf_const(magn=0.7)], G.lik_gaussian(sigma=0.05))
    l64f, g64f = _fit_grad_abi(gp(), x, y, "fp64", True)
    l64, g64 = _fit_grad_abi(gp(), x, y, "fp64", False)
    assert abs(l64f - l64) <= 1e-13 * abs(l64) and relmax(g64f, g64) < 1e-12
    lmf, gmf = _fit_grad_abi(gp(), x, y, "mixed", True)
    lm, gm = _fit_grad_abi(gp(), x, y, "mixed", False)
    assert abs(lmf - lm) <= 1e-10 * abs(lm)
    assert abs(lmf - l64) <= 1e-8 * abs(l64)  # the mixed path's stated bound (about 1.5e-9 here)
    assert relmax(gmf, gm) < 1e-9
    assert relmax(gmf, g64) < 1e-7
