"""Generate the golden fixtures of tests/golden from the oracle.

The reference (R gplite 0.13.0) cannot run in this environment and ships no
vectors, so the fixtures freeze the oracle's outputs on numpy-seeded inputs
that follow the workloads' stated shapes: a regression pin for the oracle and
the checked values for the CUDA library. Run from the repository root:
    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from oracle import gplite_ref as R  # noqa: E402


def c1():
    """1D regression, n=200, cf_sexp(0.3, 1) + lik_gaussian(0.1), pred on 300 grid points."""
    rng = np.random.default_rng(1)
    n = 200
    x = rng.standard_normal(n)
    y = np.sin(3 * x) * np.exp(-np.abs(x)) + 0.1 * rng.standard_normal(n)
    xt = np.linspace(-4, 4, 300)
    gp = R.gp_init([R.cf("sexp", lscale=0.3, magn=1.0)], R.lik("gaussian", sigma=0.1))
    gp = R.gp_fit(gp, x, y)
    p = R.gp_pred(gp, xt, var=True)
    loo = R.gp_loo(gp, x, y)
    return dict(x=x, y=y, xt=xt, lml=gp.fit["log_evidence"], alpha=gp.fit["alpha"],
                fmean=gp.fit["fmean"], mean=p["mean"], var=p["var"], loos=loo["loos"],
                energy=R.gp_energy(gp))


def c3_small():
    """Bernoulli classification (logit), n=256, d=4, cf_sexp(0.5, 2): Laplace and EP + LOO."""
    rng = np.random.default_rng(3)
    n, d = 256, 4
    x = rng.standard_normal((n, d))
    K = R.eval_cf([R.cf("sexp", lscale=0.5, magn=2.0)], x, x) + 1e-6 * np.eye(n)
    f = np.linalg.cholesky(K) @ rng.standard_normal(n)
    y = (rng.uniform(size=n) < 1 / (1 + np.exp(-f))).astype(np.float64)
    out = dict(x=x, y=y)
    gp = R.gp_fit(R.gp_init([R.cf("sexp", lscale=0.5, magn=2.0)], R.lik("bernoulli"),
                            approx=R.approx_laplace(tol=1e-6)), x, y)
    out.update(la_lml=gp.fit["log_evidence"], la_fmean=gp.fit["fmean"], la_iters=gp.fit["iters"],
               la_loos=R.gp_loo(gp, x, y)["loos"])
    gp = R.gp_fit(R.gp_init([R.cf("sexp", lscale=0.5, magn=2.0)], R.lik("bernoulli"),
                            approx=R.approx_ep(damping=0.9)), x, y)
    out.update(ep_lml=gp.fit["log_evidence"], ep_fmean=gp.fit["fmean"], ep_iters=gp.fit["iters"],
               ep_loos=R.gp_loo(gp, x, y)["loos"])
    return out


def main():
    np.savez_compressed(os.path.join(HERE, "c1_gauss_n200.npz"), **c1())
    np.savez_compressed(os.path.join(HERE, "c3_bernoulli_n256.npz"), **c3_small())
    x, w = R.gauss_hermite_points(11)
    np.savez_compressed(os.path.join(HERE, "gh.npz"), x11=x, w11=w,
                        x15=R.gauss_hermite_points(15)[0], w15=R.gauss_hermite_points(15)[1])
    print("written")


if __name__ == "__main__":
    main()
