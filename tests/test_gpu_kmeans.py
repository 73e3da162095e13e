"""Inducing inputs by k-means (get_inducing, R/gp_fit.R:192-236) on the device:
Lloyd iterations equal a NumPy restatement from the same initial centres,
well-separated blobs are recovered, and method_fitc without inducing inputs
fits with the selected centres exactly as when they are passed in."""
import warnings

import numpy as np
import pytest

import gplite_gb300 as G
from gplite_gb300.gp import get_inducing, kmeans

pytestmark = pytest.mark.gpu


def lloyd(x, init, max_iter=10):
    """Lloyd's algorithm as the device runs it: nearest centre (ties to the lower index),
    centre = mean of its points in point order, empty clusters keep their centre."""
    c = init.copy()
    assign = np.full(len(x), -1)
    for it in range(1, max_iter + 1):
        d2 = ((x[:, None, :] - c[None, :, :]) ** 2).sum(-1)
        a = d2.argmin(1)
        if np.array_equal(a, assign):
            return c, it
        assign = a
        for j in range(len(c)):
            pts = x[a == j]
            if len(pts):
                c[j] = pts.sum(0) / len(pts)
    return c, max_iter


def test_kmeans_matches_lloyd_restatement():
    rng = np.random.default_rng(0)
    x = rng.standard_normal((5000, 3))
    init = x[rng.choice(5000, 40, replace=False)]
    c, it, wss = kmeans(x, 40, init, max_iter=10)
    cr, itr = lloyd(x, init, 10)
    assert it == itr
    assert np.max(np.abs(c - cr)) < 1e-12
    d2 = ((x[:, None, :] - c[None, :, :]) ** 2).sum(-1).min(1)
    assert abs(wss - d2.sum()) <= 1e-9 * d2.sum()


def test_kmeans_recovers_blobs():
    rng = np.random.default_rng(1)
    centres = np.array([[-5.0, 0.0], [5.0, 0.0], [0.0, 6.0]])
    x = np.vstack([c + 0.3 * rng.standard_normal((400, 2)) for c in centres])
    init = x[[0, 400, 800]]
    c, it, _ = kmeans(x, 3, init, max_iter=20)
    for ct in centres:
        assert np.min(np.linalg.norm(c - ct, axis=1)) < 0.1


def test_fitc_without_inducing_inputs():
    rng = np.random.default_rng(2)
    n = 4000
    x = rng.uniform(-2, 2, (n, 2))
    y = np.sin(2 * x[:, 0]) + 0.1 * rng.standard_normal(n)
    gp = G.gp_init(G.cf_sexp(lscale=0.8), G.lik_gaussian(sigma=0.1), method=G.method_fitc(num_inducing=48))
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        gp = G.gp_fit(gp, x, y)
    z = gp.method.inducing
    assert z.shape == (48, 2)
    assert np.all(z.min(0) > -2.1) and np.all(z.max(0) < 2.1)
    g2 = G.gp_fit(G.gp_init(G.cf_sexp(lscale=0.8), G.lik_gaussian(sigma=0.1), method=G.method_fitc(inducing=z)),
                  x, y)
    assert g2.fit["log_evidence"] == gp.fit["log_evidence"]
    # binned placement along the first input: the counts per bin follow the reference's split
    gb = G.gp_init(G.cf_sexp(lscale=0.8), G.lik_gaussian(sigma=0.1),
                   method=G.method_fitc(num_inducing=30, bin_along=0, bin_count=4))
    zb = get_inducing(gb, x)
    assert zb.shape == (30, 2)
