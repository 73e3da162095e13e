"""gp_draw (R/gp_draw.R) on the device: the predictive covariance against the
oracle's formula, the draws as an exact function of the standard normals, and
their moments (R's random stream cannot be reproduced, as in the reference's
own test_pred.R:125-142 the check is statistical)."""
import numpy as np
import pytest
from scipy import linalg as sla

import gplite_gb300 as G
from oracle import gplite_ref as R

pytestmark = pytest.mark.gpu


def _setup(n=300, seed=0):
    rng = np.random.default_rng(seed)
    x = rng.uniform(-2, 2, (n, 2))
    y = np.sin(2 * x[:, 0]) * np.cos(x[:, 1]) + 0.1 * rng.standard_normal(n)
    xt = rng.uniform(-2, 2, (70, 2))
    gp = G.gp_fit(G.gp_init(G.cf_matern32(lscale=0.8, magn=1.2), G.lik_gaussian(sigma=0.1)), x, y)
    og = R.gp_fit(R.gp_init([R.cf("matern32", lscale=0.8, magn=1.2)], R.lik("gaussian", sigma=0.1)), x, y)
    return gp, og, x, y, xt


def _oracle_cov(og, x, xt, jitter=1e-6):
    Kt = R.eval_cf(og.cfs, xt, x)
    Ktt = R.eval_cf(og.cfs, xt, xt)
    aux = sla.solve_triangular(og.fit["C_chol"], Kt.T, lower=True)
    return Kt @ og.fit["alpha"], Ktt - aux.T @ aux + jitter * np.eye(len(xt))


def test_predictive_covariance_matches_oracle():
    gp, og, x, y, xt = _setup()
    mean, cov = G.gp_pred_cov(gp, xt)
    m_ref, c_ref = _oracle_cov(og, x, xt)
    assert np.max(np.abs(mean - m_ref)) <= 1e-10 * np.max(np.abs(m_ref))
    assert np.max(np.abs(cov - c_ref)) <= 1e-10 * np.max(np.abs(c_ref))
    # the diagonal is gp_pred's variance plus the jitter
    p = G.gp_pred(gp, xt, var=True)
    assert np.max(np.abs(np.diag(cov) - 1e-6 - p["var"])) <= 1e-10 * np.max(np.abs(c_ref))


def test_draws_are_mean_plus_cholesky_times_normals():
    gp, og, x, y, xt = _setup()
    s = G.gp_draw(gp, xt, draws=5, transform=False, seed=11)
    m_ref, c_ref = _oracle_cov(og, x, xt)
    z = np.random.default_rng(11).standard_normal((len(xt), 5))
    ref = m_ref[:, None] + np.linalg.cholesky(c_ref) @ z
    assert s.shape == (len(xt), 5)
    assert np.max(np.abs(s - ref)) <= 1e-8 * np.max(np.abs(ref))
    # marginal draws use the variances only
    sm = G.gp_draw(gp, xt, draws=3, transform=False, marginal=True, seed=5)
    p = G.gp_pred(gp, xt, var=True)
    zm = np.random.default_rng(5).standard_normal((len(xt), 3))
    assert np.allclose(sm, p["mean"][:, None] + np.sqrt(p["var"])[:, None] * zm, rtol=0, atol=1e-12)


def test_draw_moments_and_prior_and_targets():
    gp, og, x, y, xt = _setup()
    s = G.gp_draw(gp, xt[:20], draws=20000, transform=False, seed=1)
    mean, cov = G.gp_pred_cov(gp, xt[:20])
    sd = np.sqrt(np.diag(cov))
    assert np.all(np.abs(s.mean(1) - mean) < 5 * sd / np.sqrt(20000))
    assert np.allclose(s.var(1), np.diag(cov), rtol=0.05)
    # prior draws of an unfitted gp: zero mean, K(xt, xt) + jitter
    g0 = G.gp_init(G.cf_sexp(lscale=0.5, magn=2.0), G.lik_gaussian(sigma=0.1))
    s0 = G.gp_draw(g0, xt[:10], draws=20000, transform=False, seed=2)
    assert np.all(np.abs(s0.mean(1)) < 5 * 2.0 / np.sqrt(20000))
    assert np.allclose(s0.var(1), 4.0, rtol=0.05)
    # transform / target for non-Gaussian likelihoods
    rng = np.random.default_rng(3)
    yb = (rng.uniform(size=len(x)) < 0.5).astype(float)
    gb = G.gp_fit(G.gp_init(G.cf_sexp(lscale=0.7), G.lik_bernoulli()), x, yb)
    pb = G.gp_draw(gb, xt, draws=4, seed=4)
    assert np.all((pb > 0) & (pb < 1))
    tb = G.gp_draw(gb, xt, draws=4, target=True, seed=4)
    assert set(np.unique(tb)) <= {0.0, 1.0}


def test_fitc_predictive_covariance_matches_oracle_and_draws():
    """gp_pred_post.method_fitc(cov = TRUE) (R/gp_pred.R:263-276) on the device against a
    restatement of the same expression from the oracle's FITC fit; its diagonal equals
    the predictive variance; draws through it have the right moments."""
    import warnings

    import numpy as np
    from scipy import linalg as sla

    import gplite_gb300 as G
    from oracle import gplite_ref as R
    from helpers import oracle_gp
    rng = np.random.default_rng(21)
    n, M, m = 400, 20, 25
    x = rng.uniform(-3, 3, (n, 2))
    z = rng.uniform(-3, 3, (M, 2))
    xt = rng.uniform(-3, 3, (m, 2))
    y = np.sin(x[:, 0]) + 0.3 * x[:, 1] + 0.2 * rng.standard_normal(n)
    gp = G.gp_init([G.cf_sexp(lscale=1.2)], G.lik_gaussian(sigma=0.2), method=G.method_fitc(inducing=z))
    og = oracle_gp(gp)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        gp = G.gp_fit(gp, x, y)
        og = R.gp_fit(og, x, y)
    mean, cov = G.gp_pred_cov(gp, xt)
    # the oracle: prior_cov - t(A2) (A1 inv_lemma_solve(C_inv, t(A1))) A2 + jitter I
    Lz = og.fit["Kz_chol"]
    A1 = sla.solve_triangular(Lz, og.fit["Kxz"].T, lower=True)
    A2 = sla.solve_triangular(Lz, R.eval_cf(og.cfs, xt, z).T, lower=True)
    Dt = R.eval_cf(og.cfs, xt, xt, diag_only=True) - (A2 ** 2).sum(0)
    prior = A2.T @ A2 + np.diag(Dt)
    ref = prior - A2.T @ (A1 @ R.inv_lemma_solve(og.fit["C_inv"], A1.T)) @ A2 + 1e-6 * np.eye(m)
    po = R.gp_pred(og, xt, var=True)
    assert np.max(np.abs(mean - po["mean"])) <= 1e-9 * np.max(np.abs(po["mean"]))
    assert np.max(np.abs(cov - ref)) <= 1e-9 * np.max(np.abs(ref))
    assert np.max(np.abs(np.diag(cov) - 1e-6 - po["var"])) <= 1e-9 * np.max(np.abs(po["var"]))
    f = G.gp_draw(gp, xt, draws=20000, transform=False, seed=3)
    assert np.max(np.abs(f.mean(1) - mean)) < 5 * np.sqrt(np.max(np.diag(cov)) / 20000)
    assert np.max(np.abs(np.cov(f) - cov)) < 0.05 * np.max(np.abs(cov))


def test_monte_carlo_loo_matches_oracle_with_the_same_normals():
    """gp_loo(quadrature = FALSE) (R/gp_loo.R:97-103): with the same normals the device
    and the oracle agree to rounding; with many draws the Monte Carlo estimate
    approaches the Gauss-Hermite one."""
    import warnings

    import numpy as np

    import gplite_gb300 as G
    from oracle import gplite_ref as R
    from helpers import oracle_gp
    rng = np.random.default_rng(22)
    n = 80
    x = rng.uniform(-3, 3, n)
    y = (rng.uniform(size=n) < 1 / (1 + np.exp(-2 * np.sin(x)))).astype(float)
    for ap in (G.approx_laplace(), G.approx_ep()):
        gp = G.gp_init(G.cf_sexp(lscale=1.0, magn=1.5), G.lik_bernoulli(), approx=ap)
        og = oracle_gp(gp)
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            gp = G.gp_fit(gp, x, y)
            og = R.gp_fit(og, x, y)
        lo = G.gp_loo(gp, x, y, quadrature=False, draws=3000, seed=5)
        zz = np.random.default_rng(5).standard_normal((n, 3000))
        ro = R.gp_loo(og, x, y, z=zz)
        assert np.max(np.abs(lo["loos"] - ro["loos"])) <= 1e-9 * np.max(np.abs(ro["loos"]))
        gh = G.gp_loo(gp, x, y)
        big = G.gp_loo(gp, x, y, quadrature=False, draws=200000, seed=6)
        assert abs(big["loo"] - gh["loo"]) < 0.02 * abs(gh["loo"])
