"""method_rf / method_rbf on the device against the oracle's restatement of the
reference's feature maps and weight-space Laplace iteration (R/cf.R:532-817,
R/laplace.R:241-266, 327-355, R/gp_pred.R:186-200, 298-318, R/gp_draw.R:87-169).

Both sides draw the frequencies / centres from numpy's generator seeded with the
method's seed, in the reference's shapes and order, so the feature maps agree.
Tolerances: 1e-10 relative on the evidence, relative to max(|evidence|, n) (the
reference's expression adds n/2 log(2 pi) to terms of similar size, so the evidence
can be much smaller than its terms); 1e-9 of the largest entry for latent
means, weights, predictions and draws (the features pass through cos / sin / erf /
exp, whose device and libm values differ by an ulp, and the Gram matrix sums n of
them)."""
import warnings

import numpy as np
import pytest

import gplite_gb300 as G
from gplite_gb300 import _lib as L
from oracle import gplite_ref as R
from helpers import oracle_gp

pytestmark = pytest.mark.gpu


def relmax(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


def data(lik, n=120, d=2, seed=3):
    rng = np.random.default_rng(seed)
    x = rng.uniform(-2, 2, (n, d))
    f = np.sin(1.5 * x[:, 0]) + 0.5 * x[:, -1]
    if lik == "gaussian":
        return x, f + 0.2 * rng.standard_normal(n), None
    if lik == "poisson":
        return x, rng.poisson(np.exp(f)).astype(float), None
    return x, (rng.uniform(size=n) < 1 / (1 + np.exp(-2 * f))).astype(float), None


def make_lik(kind):
    return {"gaussian": G.lik_gaussian(sigma=0.3), "poisson": G.lik_poisson(),
            "bernoulli": G.lik_bernoulli()}[kind]


CFS = {
    "sexp": lambda: [G.cf_sexp(lscale=0.8, magn=1.2)],
    "nn": lambda: [G.cf_nn(sigma0=0.7, sigma=1.5, magn=1.1)],
    "periodic": lambda: [G.cf_periodic(period=2.5)],
    "sum": lambda: [G.cf_const(magn=0.4), G.cf_lin(magn=0.3), G.cf_sexp(lscale=0.6, magn=0.9)],
    "prod": lambda: [G.cf_sexp(lscale=0.9, vars=[0]) * G.cf_nn(vars=[1], sigma=1.2)],
}


def fit_both(cfs, lik, method, x, y):
    gp = G.gp_init(cfs, make_lik(lik), method=method)
    og = oracle_gp(gp)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        gp = G.gp_fit(gp, x, y)
        og = R.gp_fit(og, x, y)
    return gp, og


@pytest.mark.parametrize("lik", ["gaussian", "poisson", "bernoulli"])
@pytest.mark.parametrize("cf", list(CFS))
def test_rf_fit_pred_loo_draw_match_oracle(cf, lik):
    x, y, _ = data(lik)
    xt = np.random.default_rng(9).uniform(-2.5, 2.5, (37, 2))
    gp, og = fit_both(CFS[cf](), lik, G.method_rf(num_basis=24), x, y)
    assert gp.fit["iters"] == og.fit["iters"]
    assert abs(gp.fit["log_evidence"] - og.fit["log_evidence"]) <= 1e-10 * max(abs(og.fit["log_evidence"]), len(y))
    assert relmax(G.model_field(gp, "fmean"), og.fit["fmean"]) < 1e-9
    assert relmax(G.model_field(gp, "wmean"), og.fit["wmean"]) < 1e-9
    assert relmax(G.model_field(gp, "wcov"), og.fit["wcov"]) < 1e-9
    p, po = G.gp_pred(gp, xt, var=True), R.gp_pred(og, xt, var=True)
    assert relmax(p["mean"], po["mean"]) < 1e-9
    assert relmax(p["var"], po["var"]) < 1e-9
    lo, loo = G.gp_loo(gp, x, y), R.gp_loo(og, x, y)
    assert relmax(lo["loos"], loo["loos"]) < 1e-9
    # posterior draws in weight space with the same standard normals
    ks = int(sum(gp.method.num_basis))
    s = G.gp_draw(gp, xt, draws=3, seed=5, transform=False)
    z = np.asfortranarray(np.random.default_rng(5).standard_normal((ks, 3)))
    assert relmax(s, R.gp_draw_rf(og, xt, z)) < 1e-9


@pytest.mark.parametrize("cf", ["sexp", "periodic", "sum"])
def test_rbf_fit_pred_match_oracle(cf):
    x, y, _ = data("poisson")
    xt = np.random.default_rng(9).uniform(-2.5, 2.5, (29, 2))
    gp, og = fit_both(CFS[cf](), "poisson", G.method_rbf(num_basis=20), x, y)
    assert gp.fit["iters"] == og.fit["iters"]
    assert abs(gp.fit["log_evidence"] - og.fit["log_evidence"]) <= 1e-10 * max(abs(og.fit["log_evidence"]), len(y))
    p, po = G.gp_pred(gp, xt, var=True), R.gp_pred(og, xt, var=True)
    assert relmax(p["mean"], po["mean"]) < 1e-9 and relmax(p["var"], po["var"]) < 1e-9
    assert relmax(G.gp_loo(gp, x, y)["loos"], R.gp_loo(og, x, y)["loos"]) < 1e-9


def test_rf_group_selection_and_prior():
    """cfind selects a covariance function's features and weights (get_weight_inds,
    R/gp.R:235-262); an unfitted model predicts and draws from the weight prior."""
    x, y, _ = data("gaussian")
    xt = np.random.default_rng(2).uniform(-2, 2, (15, 2))
    cfs = CFS["sum"]()
    gp0 = G.gp_init(cfs, make_lik("gaussian"), method=G.method_rf(num_basis=16))
    og0 = oracle_gp(gp0)
    pv, pvo = G.gp_pred(gp0, xt, var=True), R.gp_pred(og0, xt, var=True)
    assert np.all(pv["mean"] == 0) and relmax(pv["var"], pvo["var"]) < 1e-12
    s0 = G.gp_draw(gp0, xt, draws=2, seed=1, transform=False)
    ks = int(sum(G.gp.check_num_basis(cfs, gp0.method.num_basis, 2)))
    z = np.asfortranarray(np.random.default_rng(1).standard_normal((ks, 2)))
    assert relmax(s0, R.gp_draw_rf(og0, xt, z)) < 1e-12
    gp, og = fit_both(cfs, "gaussian", G.method_rf(num_basis=16), x, y)
    for cfind in ([2], [0, 1]):
        p, po = G.gp_pred(gp, xt, var=True, cfind=cfind), R.gp_pred(og, xt, var=True, cfind=cfind)
        assert relmax(p["mean"], po["mean"]) < 1e-9 and relmax(p["var"], po["var"]) < 1e-9
        ks = int(sum(gp.method.num_basis[k] for k in cfind))
        s = G.gp_draw(gp, xt, draws=2, seed=3, cfind=cfind, transform=False)
        z = np.asfortranarray(np.random.default_rng(3).standard_normal((ks, 2)))
        assert relmax(s, R.gp_draw_rf(og, xt, z, cfind=cfind)) < 1e-9


def test_rf_refusals():
    """The reference's errors: Matern random features, an odd count for cf_sexp, EP,
    and (new functionality) no device gradient for rf."""
    x, y, _ = data("gaussian")
    with pytest.raises(ValueError):
        G.gp_fit(G.gp_init(G.cf_matern32(), G.lik_gaussian(), method=G.method_rf(num_basis=10)), x, y)
    with pytest.raises((ValueError, L.GpgpError)):
        G.gp_fit(G.gp_init(G.cf_sexp(), G.lik_gaussian(), method=G.method_rf(num_basis=11)), x, y)
    xb, yb, _ = data("bernoulli")
    with pytest.raises(ValueError):
        G.gp_fit(G.gp_init(G.cf_sexp(), G.lik_bernoulli(), method=G.method_rf(num_basis=10),
                           approx=G.approx_ep()), xb, yb)
    gp = G.gp_fit(G.gp_init(G.cf_sexp(), G.lik_gaussian(), method=G.method_rf(num_basis=10)), x, y)
    with pytest.raises(Exception):
        G.gp_energy_grad(gp)
