"""Host-side logic of the product package against the oracle (CPU only):
parameter packing, priors, translation of covariance specs to the C ABI."""
import copy
import math

import numpy as np

import gplite_gb300 as G
from gplite_gb300 import _lib as L
from gplite_gb300.gp import kernel_struct, lpdf_prior
from oracle import gplite_ref as R
from helpers import basic_models, oracle_gp


def test_param_names_and_values_match_oracle():
    for cfs in basic_models():
        gp = G.gp_init(cfs, G.lik_gaussian())
        n1, p1 = G.get_param(gp)
        n2, p2 = R.get_param(oracle_gp(gp))
        assert n1 == n2
        assert np.array_equal(p1, p2)


def test_set_param_roundtrip_and_refit_flag():
    rng = np.random.default_rng(3)
    for cfs in basic_models():
        gp = G.gp_init(cfs, G.lik_gaussian())
        _, p = G.get_param(gp)
        q = p + rng.standard_normal(len(p))
        G.set_param(gp, q)
        assert not gp.fitted
        assert np.allclose(G.get_param(gp)[1], q, rtol=0, atol=1e-14)


def test_priors_match_oracle():
    cfs = [G.cf_sexp(prior_lscale=G.prior_lognormal(0.5, 2.0), prior_magn=G.prior_half_t(3, 2)),
           G.cf_nn(), G.cf_periodic(prior_period=G.prior_fixed())]
    gp = G.gp_init(cfs, G.lik_gaussian(prior_sigma=G.prior_lognormal()))
    assert abs(lpdf_prior(gp) - R.lpdf_prior(oracle_gp(gp))) < 1e-12
    names, _ = G.get_param(gp)
    assert "cf_periodic.period" not in names


def test_prior_gradients_by_finite_difference():
    for pr in [G.prior_lognormal(0.3, 1.7), G.prior_half_t(4, 2.0), G.prior_half_t()]:
        for th in (-1.0, 0.2, 1.5):
            h = 1e-6
            fd = (pr.lpdf(th + h) - pr.lpdf(th - h)) / (2 * h)
            assert abs(fd - pr.dlpdf(th)) < 1e-7


def test_kernel_struct_translation():
    c = G.cf_sexp(vars=[1], lscale=0.7, magn=2.0) * G.cf_lin(vars=[0])
    cfs = [c, G.cf_periodic(period=3.0, cf_base=G.cf_matern52(lscale=0.4)), G.cf_const(magn=0.5)]
    k = kernel_struct(cfs, 3)
    assert k.nterms == 4 and k.ngroups == 3
    t = k.term
    assert (t[0].kind, t[0].group, t[0].nvars, t[0].vars[0]) == (L.CF_KIND["sexp"], 0, 1, 1)
    assert (t[1].kind, t[1].group) == (L.CF_KIND["lin"], 0)
    assert (t[2].kind, t[2].group, t[2].periodic, t[2].period) == (L.CF_KIND["matern52"], 1, 1, 3.0)
    assert math.isclose(t[2].lscale, 0.4)
    assert (t[3].kind, t[3].group, t[3].magn) == (L.CF_KIND["const"], 2, 0.5)


def test_gp_init_errors_like_reference():
    import pytest
    with pytest.raises(ValueError):
        G.gp_init(G.cf_sexp(), G.lik_gaussian(), approx=G.approx_ep())
    with pytest.raises(ValueError):
        G.approx_ep(damping=1.0)
    gp = G.gp_init(G.cf_sexp(), G.lik_gaussian())
    with pytest.raises(RuntimeError):
        G.gp_energy(gp)


def test_gauss_hermite_host_matches_oracle():
    from gplite_gb300.gp import gauss_hermite_points
    for q in (7, 11, 15):
        a, wa = gauss_hermite_points(q)
        b, wb = R.gauss_hermite_points(q)
        assert np.allclose(a, b, rtol=0, atol=1e-13) and np.allclose(wa, wb, rtol=1e-12)


def test_stale_fit_is_refused_before_any_device_call():
    """test_pred.R:85-120 / test_loo.R:114-144: after set_param, gp_pred, gp_draw, gp_loo
    and gp_energy refuse a model that still holds the old posterior, until it is refitted;
    the check is host logic and runs before any device work."""
    import pytest
    gp = G.gp_init(G.cf_sexp(), G.lik_gaussian())
    gp.fit = {"type": "analytic"}  # a posterior from an earlier fit
    _, p = G.get_param(gp)
    p[0] = 0.0
    G.set_param(gp, p)
    x = np.zeros((3, 1))
    for call in (lambda: G.gp_pred(gp, x, var=True), lambda: G.gp_pred(gp, x),
                 lambda: G.gp_draw(gp, x, draws=1), lambda: G.gp_loo(gp, x, np.zeros(3)),
                 lambda: G.gp_energy(gp)):
        with pytest.raises(RuntimeError, match="refit"):
            call()


def test_fit_with_gradient_needs_gaussian_full_before_any_device_call():
    """gp_fit(..., grad=True) (the fit and its energy gradient in one call) exists for
    lik_gaussian with method_full only, like gp_energy_grad; other models are refused on
    the host, before a context or the library is touched."""
    import pytest
    x, y = np.zeros((4, 1)), np.zeros(4)
    for gp in (G.gp_init(G.cf_sexp(), G.lik_bernoulli()),
               G.gp_init(G.cf_sexp(), G.lik_gaussian(), method=G.method_fitc(num_inducing=2))):
        with pytest.raises(ValueError, match="lik_gaussian and method_full"):
            G.gp_fit(gp, x, y, grad=True)
