"""Parity of the CUDA library (through the C ABI) with the oracle, FP64 plain path.

Tolerance: 1e-10 relative on log evidence, posterior mean, posterior variance
and alpha, the bar the plain path is held to; covariance matrices to 1e-12.
Cases restate the reference's tests (tests/testthat/test_basic.R,
test_normalization.R, test_loo.R, test_pred.R) with numpy-seeded data.
"""
import copy
import os
import warnings

import numpy as np
import pytest

import gplite_gb300 as G
from gplite_gb300 import _lib as L
from oracle import gplite_ref as R
from helpers import basic_models, close, oracle_gp, rel_err

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")
RTOL = 1e-10


def basic_data():
    rng = np.random.default_rng(1234)
    x = rng.standard_normal(20)
    xt = rng.standard_normal(30)
    y = x ** 2 + 0.2 * rng.standard_normal(20)
    return x, xt, y


def test_cf_ffi_routines_match_oracle():
    """gpgp_cf_* replace src/cf.cpp:9-162 (incl. diag_only)."""
    rng = np.random.default_rng(0)
    lib = L.load()
    for d in (1, 3, 8):
        x1 = np.asfortranarray(rng.standard_normal((37, d)))
        x2 = np.asfortranarray(rng.standard_normal((53, d)))
        for name, fn, args in [("sexp", R.cf_sexp_c, (0.7, 1.3)), ("matern32", R.cf_matern32_c, (0.9, 0.8)),
                               ("matern52", R.cf_matern52_c, (0.4, 2.0)), ("nn", R.cf_nn_c, (1.1, 2.5, 0.7))]:
            for diag in (0, 1):
                out = np.empty(37) if diag else np.empty((37, 53), order="F")
                f = getattr(lib, "gpgp_cf_" + name)
                st = f(L.ptr(x1), 37, L.ptr(x2), 53, d, *args, diag, out.ctypes.data)
                assert st == 0
                ref = fn(x1, x2, *args, diag_only=bool(diag))
                assert close(out, ref, 1e-12, 1e-15), (name, d, diag)


def test_eval_cf_all_combinations():
    x, xt, _ = basic_data()
    for cfs in basic_models():
        G.gp.learn_scales(G.gp_init(cfs), x)
        K = G.eval_cf(cfs, xt, x)
        Kr = R.eval_cf(copy.deepcopy(cfs), xt, x)
        assert close(K, Kr, 1e-12, 1e-14), cfs
        Kd = G.eval_cf(cfs, xt, xt, diag_only=True)
        assert close(Kd, R.eval_cf(copy.deepcopy(cfs), xt, xt, diag_only=True), 1e-12, 1e-14)


def test_gaussian_fit_and_pred_all_combinations():
    """test_basic.R:64-132 at 1e-10 against the restatement."""
    x, xt, y = basic_data()
    rng = np.random.default_rng(2309)
    for cfs in basic_models():
        gp = G.gp_init(cfs, G.lik_gaussian())
        _, p0 = G.get_param(gp)
        G.set_param(gp, p0 + 0.3 * rng.standard_normal(len(p0)))
        og = oracle_gp(gp)
        gp = G.gp_fit(gp, x, y)
        og = R.gp_fit(og, x, y)
        assert rel_err(gp.fit["log_evidence"], og.fit["log_evidence"]) < RTOL, cfs
        assert close(G.model_field(gp, "alpha"), og.fit["alpha"], 1e-9, 1e-10)
        p = G.gp_pred(gp, xt, var=True)
        po = R.gp_pred(og, xt, var=True)
        assert close(p["mean"], po["mean"], RTOL, 1e-11), cfs
        assert close(p["var"], po["var"], 1e-9, 1e-11), cfs


@pytest.mark.parametrize("n", [1, 2, 7, 33, 63, 64, 65, 130, 257])
def test_odd_sizes(n):
    """Every tile-edge path of the blocked kernels (NB = 64, tiles of 64)."""
    rng = np.random.default_rng(n)
    x = rng.uniform(-2, 2, (n, 2))
    y = np.sin(x[:, 0]) + 0.1 * rng.standard_normal(n)
    xt = rng.uniform(-2, 2, (n + 3, 2))
    gp = G.gp_init([G.cf_sexp(lscale=0.8), G.cf_const(0.5)], G.lik_gaussian(sigma=0.2))
    og = oracle_gp(gp)
    gp = G.gp_fit(gp, x, y)
    og = R.gp_fit(og, x, y)
    assert rel_err(gp.fit["log_evidence"], og.fit["log_evidence"]) < RTOL
    p, po = G.gp_pred(gp, xt, var=True), R.gp_pred(og, xt, var=True)
    assert close(p["mean"], po["mean"], RTOL, 1e-12)
    assert close(p["var"], po["var"], 1e-9, 1e-12)


def test_golden_c1():
    g = np.load(os.path.join(GOLD, "c1_gauss_n200.npz"))
    gp = G.gp_fit(G.gp_init(G.cf_sexp(lscale=0.3, magn=1.0), G.lik_gaussian(sigma=0.1)), g["x"], g["y"])
    assert rel_err(gp.fit["log_evidence"], float(g["lml"])) < RTOL
    assert rel_err(G.gp_energy(gp), float(g["energy"])) < RTOL
    p = G.gp_pred(gp, g["xt"], var=True)
    assert close(p["mean"], g["mean"], RTOL, 1e-12)
    assert close(p["var"], g["var"], 1e-9, 1e-12)
    loo = G.gp_loo(gp, g["x"], g["y"])
    assert close(loo["loos"], g["loos"], 1e-9, 1e-12)


@pytest.mark.parametrize("approx", ["laplace", "ep"])
def test_golden_c3_bernoulli(approx):
    g = np.load(os.path.join(GOLD, "c3_bernoulli_n256.npz"))
    ap = G.approx_laplace(tol=1e-6) if approx == "laplace" else G.approx_ep(damping=0.9)
    gp = G.gp_fit(G.gp_init(G.cf_sexp(lscale=0.5, magn=2.0), G.lik_bernoulli(), approx=ap), g["x"], g["y"])
    pre = "la_" if approx == "laplace" else "ep_"
    assert gp.fit["iters"] == int(g[pre + "iters"])
    assert rel_err(gp.fit["log_evidence"], float(g[pre + "lml"])) < 1e-9
    assert close(G.model_field(gp, "fmean"), g[pre + "fmean"], 1e-9, 1e-11)
    loo = G.gp_loo(gp, g["x"], g["y"])
    assert close(loo["loos"], g[pre + "loos"], 1e-9, 1e-11)


LIKS = [("bernoulli", "logit"), ("bernoulli", "probit"), ("binomial", "logit"), ("poisson", "log")]


@pytest.mark.parametrize("lik,link", LIKS)
@pytest.mark.parametrize("approx", ["laplace", "ep"])
def test_non_gaussian(lik, link, approx):
    """test_loo.R-style sweep: every likelihood x approximation, with LOO."""
    rng = np.random.default_rng(1234)
    n = 30
    x = rng.uniform(-3, 3, n)
    f = 2 * x - 4 if lik != "poisson" else 0.5 * x
    trials = rng.integers(1, 11, n).astype(np.float64)
    mu = 1 / (1 + np.exp(-f))
    if lik == "bernoulli":
        y = (rng.uniform(size=n) < mu).astype(np.float64)
    elif lik == "binomial":
        y = rng.binomial(trials.astype(int), mu).astype(np.float64)
    else:
        y = rng.poisson(np.exp(f)).astype(np.float64)
    mk = {"bernoulli": G.lik_bernoulli, "binomial": G.lik_binomial, "poisson": G.lik_poisson}[lik]
    ap = G.approx_laplace() if approx == "laplace" else G.approx_ep(damping=0.8)
    offset = 0.1 * rng.standard_normal(n)
    for cf in [G.cf_sexp(lscale=1.0), G.cf_lin(), G.cf_const(), G.cf_nn(), G.cf_periodic()]:
        gp = G.gp_init(cf, mk(link), approx=ap)
        og = oracle_gp(gp)
        kw = dict(trials=trials if lik == "binomial" else None, offset=offset)
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            gp = G.gp_fit(gp, x, y, **kw)
            og = R.gp_fit(og, x, y, **kw)
        assert gp.fit["iters"] == og.fit["iters"], (lik, approx, cf)
        assert close(gp.fit["log_evidence"], og.fit["log_evidence"], 1e-9, 1e-12), (lik, approx, cf)
        assert close(G.model_field(gp, "fmean"), og.fit["fmean"], 1e-9, 1e-11)
        loo = G.gp_loo(gp, x, y, quad_order=7)
        lo = R.gp_loo(og, x, y, quad_order=7, **kw)
        assert not np.any(np.isnan(loo["loos"]))
        assert close(loo["loos"], lo["loos"], 1e-8, 1e-10), (lik, approx, cf)


def test_refit_required_after_set_param():
    """test_loo.R:114-144 / test_pred.R:85-120: pred and loo error until refit."""
    x, xt, y = basic_data()
    gp = G.gp_fit(G.gp_init(G.cf_sexp(), G.lik_gaussian()), x, y)
    G.gp_pred(gp, xt, var=True)
    _, p = G.get_param(gp)
    p[0] = 0.0
    G.set_param(gp, p)
    with pytest.raises(RuntimeError):
        G.gp_pred(gp, xt)
    with pytest.raises(RuntimeError):
        G.gp_loo(gp, x, y)
    gp = G.gp_fit(gp, x, y)
    assert np.all(np.isfinite(G.gp_loo(gp, x, y)["loos"]))


def test_prior_prediction_unfitted():
    x, xt, y = basic_data()
    gp = G.gp_init([G.cf_sexp(), G.cf_lin()], G.lik_gaussian())
    p = G.gp_pred(gp, xt, var=True)
    assert np.all(p["mean"] == 0)
    assert close(p["var"], R.eval_cf(copy.deepcopy(gp.cfs), xt, xt, diag_only=True), 1e-12)


def test_cfind_and_transform_quantiles():
    x, xt, y = basic_data()
    gp = G.gp_init([G.cf_sexp(), G.cf_lin()], G.lik_gaussian())
    og = oracle_gp(gp)
    gp, og = G.gp_fit(gp, x, y), R.gp_fit(og, x, y)
    for cfind in ([0], [1]):
        p, po = G.gp_pred(gp, xt, var=True, cfind=cfind), R.gp_pred(og, xt, var=True, cfind=cfind)
        assert close(p["mean"], po["mean"], RTOL, 1e-12) and close(p["var"], po["var"], 1e-9, 1e-12)
    gb = G.gp_init(G.cf_sexp(lscale=1.0), G.lik_bernoulli())
    ob = oracle_gp(gb)
    yb = (x > 0).astype(float)
    gb, ob = G.gp_fit(gb, x, yb), R.gp_fit(ob, x, yb)
    p = G.gp_pred(gb, xt, quantiles=[0.1, 0.9], transform=True)
    po = R.gp_pred(ob, xt, quantiles=[0.1, 0.9], transform=True)
    assert close(p["mean"], po["mean"], 1e-9, 1e-12) and close(p["quantiles"], po["quantiles"], 1e-9, 1e-12)


def test_not_positive_definite_is_an_error():
    """chol failure in method_full is an R error (R/laplace.R:28); here NotPositiveDefinite."""
    x, _, y = basic_data()
    gp = G.gp_init(G.cf_sexp(), G.lik_gaussian(sigma=0.01))
    with pytest.raises(np.linalg.LinAlgError):
        G.gp_fit(gp, x, y, jitter=-10.0)
    # the context stays usable
    gp = G.gp_fit(G.gp_init(G.cf_sexp(), G.lik_gaussian()), x, y)
    assert np.isfinite(gp.fit["log_evidence"])


def test_energy_gradient_matches_oracle():
    """The gradient has no counterpart in the reference (it optimises with Nelder-Mead,
    R/gp_optim.R:76-94). The oracle's gradient (analytic covariance derivatives pinned by
    complex-step differentiation of eval_cf, the trace formula by finite differences of the
    oracle energy, both in tests/test_oracle.py) holds the device gradient to 1e-10
    relative per component (components below 1e-10 of the largest are held absolutely).
    One-ulp input changes move the oracle's own gradient by <= 1.2e-13 here."""
    rng = np.random.default_rng(5)
    n = 150
    x = rng.uniform(-1, 1, (n, 3))
    y = np.sin(2 * x[:, 0]) + x[:, 1] ** 2 + 0.05 * rng.standard_normal(n)
    for cfs in ([G.cf_matern52(lscale=0.7), G.cf_const(1.0)], [G.cf_sexp(lscale=0.5, magn=1.2)],
                [G.cf_matern32(vars=[0, 2]) * G.cf_lin(vars=[1])], [G.cf_nn(), G.cf_periodic(period=1.7)],
                [G.cf_periodic(period=0.9, cf_base=G.cf_matern52(lscale=0.8)), G.cf_lin(normalize=True)]):
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            gp = G.gp_init(cfs, G.lik_gaussian(sigma=0.1, prior_sigma=G.prior_lognormal()))
        og = oracle_gp(gp)
        gp = G.gp_fit(gp, x, y)
        og = R.gp_fit(og, x, y)
        g = G.gp_energy_grad(gp)
        go = R.gp_energy_grad(og)
        assert close(g, go, RTOL, RTOL * np.max(np.abs(go))), (cfs, g, go)


def test_energy_gradient_with_the_fit_matches_oracle():
    """gp_fit(..., grad=True) (gpgp_fit_grad): at n = 1200 (at least as many 64-tiles of
    K as SMs) the covariance pass writes K's derivative matrices beside K and the
    gradient is one pass over them; held to the oracle's gradient at 1e-10 as above,
    for kernels with a product group of a constant and a stationary term, a group of
    constants only, periodic, lin and nn terms. The evidence equals the separate
    gp_fit's (the same K)."""
    rng = np.random.default_rng(11)
    n = 1200
    x = rng.uniform(-1, 1, (n, 3))
    y = np.sin(2 * x[:, 0]) + x[:, 1] ** 2 + 0.05 * rng.standard_normal(n)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")  # products with two free magnitudes warn (R/misc.R:76)
        cases = [[G.cf_matern52(lscale=0.7), G.cf_const(1.0)], [G.cf_sexp(lscale=0.5, magn=1.2)],
                 [G.cf_const(0.8) * G.cf_matern32(lscale=0.9), G.cf_const(0.5) * G.cf_const(1.5)],
                 [G.cf_matern32(vars=[0, 2]) * G.cf_lin(vars=[1])], [G.cf_nn(), G.cf_periodic(period=1.7)],
                 [G.cf_periodic(period=0.9, cf_base=G.cf_matern52(lscale=0.8)), G.cf_lin(normalize=True)]]
        gps = [G.gp_init(cfs, G.lik_gaussian(sigma=0.1, prior_sigma=G.prior_lognormal())) for cfs in cases]
    for cfs, gp in zip(cases, gps):
        og = R.gp_fit(oracle_gp(gp), x, y)
        lml_sep = G.gp_fit(copy.deepcopy(gp), x, y).fit["log_evidence"]
        gp = G.gp_fit(gp, x, y, grad=True)
        assert gp.fit["grad_raw"] is not None
        g = G.gp_energy_grad(gp)
        go = R.gp_energy_grad(og)
        assert rel_err(gp.fit["log_evidence"], og.fit["log_evidence"]) <= RTOL
        assert abs(gp.fit["log_evidence"] - lml_sep) <= 1e-13 * abs(lml_sep)
        assert close(g, go, RTOL, RTOL * np.max(np.abs(go))), (cfs, g, go)


FITC_LIKS = [("gaussian", "laplace"), ("poisson", "laplace"), ("bernoulli", "laplace"),
             ("bernoulli", "ep"), ("poisson", "ep")]


def relmax(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


@pytest.mark.parametrize("lik,approx", FITC_LIKS)
def test_fitc_matches_oracle(lik, approx):
    """method_fitc with given inducing points (R/gp_fit.R:101-188): evidence, posterior mean,
    prediction and LOO against the restatement (test_sparse.R / test_loo.R shapes).

    Vectors are compared in the max norm relative to their largest entry (1e-9): FITC's
    solves with K_z (condition ~3e4 here) and the lemma's cancellation z/S - iDU C^-1 iDU^T z
    make single entries sensitive at ~1e-8 to one-ulp input changes (measured on the oracle
    itself), so per-entry 1e-10 would test rounding noise, not the algorithm. The LOO
    densities add one more cancellation (1/post_var - 1/V): one-ulp relative changes of x
    and z move the oracle's own max-norm LOO by 1.7e-9 .. 1.9e-8 (four seeds), so they are
    held to 5e-8."""
    rng = np.random.default_rng(7)
    n, M = 300, 24
    x = rng.uniform(-3, 3, (n, 2))
    xt = rng.uniform(-3, 3, (41, 2))
    z = rng.uniform(-3, 3, (M, 2))
    f = np.sin(x[:, 0]) + 0.5 * x[:, 1]
    if lik == "gaussian":
        y = f + 0.2 * rng.standard_normal(n)
        lk = G.lik_gaussian(sigma=0.2)
    elif lik == "poisson":
        y = rng.poisson(np.exp(f)).astype(float)
        lk = G.lik_poisson()
    else:
        y = (rng.uniform(size=n) < 1 / (1 + np.exp(-2 * f))).astype(float)
        lk = G.lik_bernoulli()
    ap = G.approx_laplace() if approx == "laplace" else G.approx_ep()
    gp = G.gp_init([G.cf_sexp(lscale=1.2, magn=1.0), G.cf_const(0.5)], lk, method=G.method_fitc(inducing=z),
                   approx=ap)
    og = oracle_gp(gp)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        gp = G.gp_fit(gp, x, y)
        og = R.gp_fit(og, x, y)
    assert gp.fit["iters"] == og.fit["iters"]
    assert rel_err(gp.fit["log_evidence"], og.fit["log_evidence"]) < 1e-10
    assert relmax(G.model_field(gp, "fmean"), og.fit["fmean"]) < 1e-9
    p, po = G.gp_pred(gp, xt, var=True), R.gp_pred(og, xt, var=True)
    assert relmax(p["mean"], po["mean"]) < 1e-9
    assert relmax(p["var"], po["var"]) < 1e-9
    loo, lo = G.gp_loo(gp, x, y), R.gp_loo(og, x, y)
    assert relmax(loo["loos"], lo["loos"]) < 5e-8


def test_fitc_method_full_agreement_at_full_inducing():
    """With every training input as an inducing point FITC's D vanishes (up to jitter) and
    its evidence approaches method_full's: a size-independent property of the lemma path."""
    rng = np.random.default_rng(11)
    n = 120
    x = rng.uniform(-2, 2, (n, 1))
    y = np.sin(2 * x[:, 0]) + 0.1 * rng.standard_normal(n)
    g1 = G.gp_fit(G.gp_init(G.cf_sexp(lscale=0.8), G.lik_gaussian(sigma=0.3)), x, y)
    g2 = G.gp_fit(G.gp_init(G.cf_sexp(lscale=0.8), G.lik_gaussian(sigma=0.3), method=G.method_fitc(inducing=x)),
                  x, y)
    assert abs(g1.fit["log_evidence"] - g2.fit["log_evidence"]) < 1e-3 * abs(g1.fit["log_evidence"])
