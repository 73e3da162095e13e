"""gp_optim driven by the device (R/gp_optim.R:63-160): Nelder-Mead as the reference
runs it, and L-BFGS on the device energy gradient, on the C1 model (n = 200,
cf_sexp + lik_gaussian). Both must reach the minimum that L-BFGS finds on the
oracle's energy and gradient: energies within tol * n (gp_optim's stopping rule,
reltol = tol with fnscale = n), parameters within tol_param."""
import copy
import warnings

import numpy as np
import pytest
from scipy.optimize import minimize

import gplite_gb300 as G
from oracle import gplite_ref as R

pytestmark = pytest.mark.gpu


def test_gp_optim_nelder_mead_and_lbfgs_reach_the_oracle_optimum():
    rng = np.random.default_rng(1)
    n = 200
    x = rng.standard_normal(n)
    y = np.sin(3 * x) * np.exp(-np.abs(x)) + 0.1 * rng.standard_normal(n)
    gp0 = lambda: G.gp_init(G.cf_sexp(lscale=0.3, magn=1.0), G.lik_gaussian(sigma=0.1))  # noqa: E731
    og0 = R.gp_init([R.cf("sexp", lscale=0.3, magn=1.0)], R.lik("gaussian", sigma=0.1))

    def o_fg(p):
        og = R.gp_fit(R.set_param(copy.deepcopy(og0), p), x, y)
        return R.gp_energy(og), R.gp_energy_grad(og)
    _, p0 = R.get_param(og0)
    ref = minimize(o_fg, p0, jac=True, method="L-BFGS-B", options=dict(ftol=1e-13, gtol=1e-10))
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        g_nm = G.gp_optim(gp0(), x, y, verbose=False)
        g_lb = G.gp_optim(gp0(), x, y, verbose=False, method="lbfgs")
    for g in (g_nm, g_lb):
        _, p = G.get_param(g)
        e = G.gp_energy(g)
        # the device energy at the returned parameters is the oracle's
        og = R.gp_fit(R.set_param(copy.deepcopy(og0), p), x, y)
        assert abs(e - R.gp_energy(og)) <= 1e-10 * abs(R.gp_energy(og))
        assert e >= ref.fun - 1e-8
        assert e - ref.fun < 1e-4 * n
        assert np.allclose(p, ref.x, atol=0.1)
    # the gradient-based run ends at the optimum itself
    assert abs(G.gp_energy(g_lb) - ref.fun) < 1e-6 * abs(ref.fun)
