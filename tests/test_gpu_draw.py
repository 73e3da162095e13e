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
