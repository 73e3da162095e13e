"""gp_optim's host logic (R/gp_optim.R:63-160): the Nelder-Mead minimiser with R's
optim defaults, the convergence probe and the restarts, on CPU. The energies come
from the oracle, so no GPU is needed; the device-driven runs are in
tests/test_gpu_optim.py."""
import copy
import warnings

import numpy as np
from scipy.optimize import minimize

from gplite_gb300.gp import _check_convergence, _nelder_mead
from oracle import gplite_ref as R


def rosenbrock(p):
    return 100.0 * (p[1] - p[0] ** 2) ** 2 + (1.0 - p[0]) ** 2


def test_nelder_mead_rosenbrock():
    """The optim() documentation example: Nelder-Mead from (-1.2, 1) reaches the
    minimum at (1, 1) within a few hundred evaluations."""
    calls = [0]

    def f(p):
        calls[0] += 1
        return rosenbrock(p)
    p, fv, conv = _nelder_mead(f, np.array([-1.2, 1.0]), reltol=1e-8, maxit=500, fnscale=1.0)
    assert conv == 0
    assert np.allclose(p, [1.0, 1.0], atol=2e-2)
    assert fv < 1e-3
    assert calls[0] <= 500


def test_nelder_mead_iteration_limit_flags_nonconvergence():
    p, fv, conv = _nelder_mead(rosenbrock, np.array([-1.2, 1.0]), reltol=1e-12, maxit=20, fnscale=1.0)
    assert conv == 1
    assert fv == rosenbrock(p)


def test_nelder_mead_fnscale_only_scales_the_stopping_rule():
    """fnscale = n (R/gp_optim.R:86-93) divides the objective: the minimiser and the
    returned (unscaled) value are those of the objective itself."""
    q = lambda p: 3.0 + ((p - np.array([0.3, -0.7, 1.1])) ** 2).sum()  # noqa: E731
    p1, f1, c1 = _nelder_mead(q, np.zeros(3), 1e-10, 2000, 1.0)
    p2, f2, c2 = _nelder_mead(q, np.zeros(3), 1e-10, 2000, 50.0)
    assert c1 == 0 and c2 == 0
    assert np.allclose(p1, [0.3, -0.7, 1.1], atol=1e-3) and np.allclose(p2, [0.3, -0.7, 1.1], atol=1e-2)
    assert abs(f1 - q(p1)) < 1e-15 and abs(f2 - q(p2)) < 1e-12


def test_check_convergence_probes():
    """check_convergence (R/gp_optim.R:127-160): +-delta per parameter; a probe that
    lowers the loss by more than tol means not converged."""
    q = lambda p: ((p - np.array([1.0, 2.0])) ** 2).sum() * 10.0  # noqa: E731
    ok, msg = _check_convergence(q, q(np.array([1.0, 2.0])), np.array([1.0, 2.0]), delta=0.1, tol=1e-2)
    assert ok and msg == "Optimization converged."
    ok, msg = _check_convergence(q, q(np.array([1.3, 2.0])), np.array([1.3, 2.0]), delta=0.1, tol=1e-2)
    assert not ok and "tol_param = 0.100000" in msg


def _c1_data(n=60, seed=1):
    rng = np.random.default_rng(seed)
    x = rng.standard_normal(n)
    y = np.sin(3 * x) * np.exp(-np.abs(x)) + 0.1 * rng.standard_normal(n)
    return x, y


def test_nelder_mead_on_the_oracle_energy_reaches_the_gradient_optimum():
    """gp_optim's Nelder-Mead (reltol = tol 1e-4, fnscale = n, maxit 500) on the
    oracle's gp_energy of the C1 model (cf_sexp + lik_gaussian) ends within
    tol * n of the minimum that L-BFGS finds with the oracle's analytic gradient."""
    x, y = _c1_data()
    n = len(y)
    gp0 = R.gp_init([R.cf("sexp", lscale=0.3, magn=1.0)], R.lik("gaussian", sigma=0.1))

    def energy(p):
        gp = R.set_param(copy.deepcopy(gp0), p)
        return R.gp_energy(R.gp_fit(gp, x, y))

    def energy_grad(p):
        gp = R.gp_fit(R.set_param(copy.deepcopy(gp0), p), x, y)
        return R.gp_energy(gp), R.gp_energy_grad(gp)
    _, p0 = R.get_param(gp0)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        p_nm, e_nm, conv = _nelder_mead(energy, p0, 1e-4, 500, n)
        r = minimize(energy_grad, p0, jac=True, method="L-BFGS-B", options=dict(ftol=1e-12, gtol=1e-9))
    assert conv == 0
    assert e_nm >= r.fun - 1e-9
    assert e_nm - r.fun < 1e-4 * n
    assert np.allclose(p_nm, r.x, atol=0.1)  # tol_param of gp_optim
    ok, _ = _check_convergence(energy, e_nm, p_nm, delta=0.1)
    assert ok
