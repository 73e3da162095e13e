"""lik_betabinom and the non-log-concave branches of the Laplace and EP iterations
(R/lik.R:332-354,400-425; R/laplace.R:40-117, R/ep.R:50-138): when some
pseudo-variance is <= 0 the sites split into good and bad ones and the final fit
solves with K + diag(V) (an LU in the reference, block elimination with the good
sites' Cholesky factor and an LU of the bad sites' Schur complement here).

Tolerances: 1e-8 relative on the evidence, and of the largest entry for latent
means, predictions and LOO densities. Beta-binomial derivatives go through
digamma, which the oracle takes from scipy and the device from its own series
(agreeing to a few ulps), and the forward-difference curvature divides their
differences by 1e-6, so the pseudo-data carry up to ~1e-9 relative noise that the
iterations pass on."""
import warnings

import numpy as np
import pytest

import gplite_gb300 as G
from gplite_gb300 import _lib as L
from oracle import gplite_ref as R
from helpers import oracle_gp

pytestmark = pytest.mark.gpu


def outlier_data(n=60, seed=2):
    rng = np.random.default_rng(seed)
    x = rng.uniform(-3, 3, n)
    N = np.full(n, 20.0)
    y = rng.binomial(20, 1 / (1 + np.exp(-1.5 * x))).astype(float)
    out = np.argsort(-np.abs(x))[:4]
    y[out] = np.where(x[out] > 0, 0.0, 20.0)  # four outliers at the ends
    return x, y, N


def relmax(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


@pytest.mark.parametrize("approx", ["laplace", "ep"])
@pytest.mark.parametrize("phi", [0.3, 1.0, 3.0])
def test_betabinom_full_matches_oracle(approx, phi):
    """phi = 0.3 makes some pseudo-variances negative (one site under Laplace, four
    under EP, checked on the oracle's fit): the split branch; 1.0 and 3.0 stay
    log-concave at these data."""
    x, y, N = outlier_data()
    xt = np.linspace(-3.5, 3.5, 17)
    ap = G.approx_laplace() if approx == "laplace" else G.approx_ep()
    gp = G.gp_init(G.cf_sexp(lscale=1.5, magn=2.0), G.lik_betabinom(phi=phi), approx=ap)
    og = oracle_gp(gp)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        gp = G.gp_fit(gp, x, y, trials=N)
        og = R.gp_fit(og, x, y, trials=N)
    if phi == 0.3:
        assert "C_lu" in og.fit and np.any(og.fit["V"] <= 0)
    assert gp.fit["iters"] == og.fit["iters"]
    assert abs(gp.fit["log_evidence"] - og.fit["log_evidence"]) <= 1e-8 * abs(og.fit["log_evidence"])
    assert relmax(G.model_field(gp, "fmean"), og.fit["fmean"]) < 1e-8
    p, po = G.gp_pred(gp, xt, var=True), R.gp_pred(og, xt, var=True)
    assert relmax(p["mean"], po["mean"]) < 1e-8
    assert relmax(p["var"], po["var"]) < 1e-8
    lo, loo = R.gp_loo(og, x, y, trials=N), G.gp_loo(gp, x, y)
    assert relmax(loo["loos"], lo["loos"]) < 1e-8


@pytest.mark.parametrize("approx", ["laplace", "ep"])
def test_betabinom_fitc_split_matches_oracle(approx):
    """The FITC split (R/laplace.R:151-231, R/ep.R:186-272): the good sites' lemma, the
    bad sites' prior through the inducing inputs, and the lemma of all sites with
    S = D + V for the final fit. Held in the max norm (FITC vectors, as in
    test_gpu_parity.py)."""
    x, y, N = outlier_data()
    z = np.linspace(-3, 3, 12)
    xt = np.linspace(-3.5, 3.5, 17)
    ap = G.approx_laplace() if approx == "laplace" else G.approx_ep()
    gp = G.gp_init(G.cf_sexp(lscale=1.5, magn=2.0), G.lik_betabinom(phi=0.3), method=G.method_fitc(inducing=z),
                   approx=ap)
    og = oracle_gp(gp)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        gp = G.gp_fit(gp, x, y, trials=N)
        og = R.gp_fit(og, x, y, trials=N)
    assert np.any(og.fit["V"] <= 0)
    assert gp.fit["iters"] == og.fit["iters"]
    assert abs(gp.fit["log_evidence"] - og.fit["log_evidence"]) <= 1e-8 * abs(og.fit["log_evidence"])
    assert relmax(G.model_field(gp, "fmean"), og.fit["fmean"]) < 1e-8
    p, po = G.gp_pred(gp, xt, var=True), R.gp_pred(og, xt, var=True)
    assert relmax(p["mean"], po["mean"]) < 1e-8 and relmax(p["var"], po["var"]) < 1e-8


def test_betabinom_mixed_precision_split_runs_in_fp64():
    """A mixed-precision fit that meets bad sites takes the same FP64 split."""
    x, y, N = outlier_data()
    gp = G.gp_init(G.cf_sexp(lscale=1.5, magn=2.0), G.lik_betabinom(phi=0.3))
    og = oracle_gp(gp)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        gm = G.gp_fit(gp, x, y, trials=N, precision="mixed")
        og = R.gp_fit(og, x, y, trials=N)
    assert abs(gm.fit["log_evidence"] - og.fit["log_evidence"]) <= 1e-8 * abs(og.fit["log_evidence"])


def test_betabinom_needs_trials():
    x, y, N = outlier_data()
    with pytest.raises(ValueError):
        G.gp_fit(G.gp_init(G.cf_sexp(), G.lik_betabinom()), x, y)


def test_digamma_series_against_scipy_through_the_likelihood():
    """The device digamma enters get_loglik_d of lik_betabinom: the pseudo-data of a
    log-concave beta-binomial fit's first Newton step match the oracle's (scipy
    digamma) to 1e-7 over a wide range of a = mu / phi, including a << 1 (the
    forward difference amplifies ulp-level differences by up to 1e6)."""
    rng = np.random.default_rng(4)
    n = 300
    x = rng.uniform(-6, 6, n)
    N = rng.integers(1, 200, n).astype(float)
    y = np.floor(N * rng.uniform(size=n))
    for phi in (1e-3, 0.05, 2.0, 50.0):
        gp = G.gp_init(G.cf_sexp(lscale=1.0, magn=3.0), G.lik_betabinom(phi=phi), approx=G.approx_laplace(maxiter=1))
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            try:
                gp = G.gp_fit(gp, x, y, trials=N)
            except L.GpgpError:
                continue  # a split whose bad-site posterior is not proper: an R error too
        z = G.model_field(gp, "z")
        V = G.model_field(gp, "V")
        zo, Vo = R.get_pseudodata_la(R.lik("betabinom", phi=phi), np.zeros(n), y, trials=N)
        assert relmax(V, Vo) < 1e-7 and relmax(z, zo) < 1e-7
