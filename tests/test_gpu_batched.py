"""Batched small GPs (gpgp_batch_*): every problem against the oracle's gp_fit,
gp_loo and gp_pred (tolerances in test_batched_matches_oracle)."""
import numpy as np
import pytest

from gplite_gb300.batch import BatchPlan, gp_fit_batched
from oracle import gplite_ref as R

pytestmark = pytest.mark.gpu


def make_problems(count, seed, nmax=300):
    rng = np.random.default_rng(seed)
    probs = []
    for i in range(count):
        n = int(np.exp(rng.uniform(np.log(3), np.log(nmax))))
        d = int(rng.integers(1, 4))
        x = rng.uniform(-2, 2, (n, d))
        y = np.sin(2 * x[:, 0]) + 0.1 * rng.standard_normal(n)
        xt = rng.uniform(-2, 2, (int(rng.integers(1, 40)), d))
        kind = ["sexp", "matern32", "matern52"][i % 3]
        probs.append(dict(x=x, y=y, xt=xt, kind=kind, lscale=float(np.exp(rng.uniform(np.log(0.2), np.log(2)))),
                          magn=float(rng.uniform(0.5, 1.5)), sigma=float(rng.uniform(0.01, 0.3))))
    return probs


def oracle_solve(p, quad_order=11, perturb=None):
    x = p["x"]
    if perturb is not None:  # one-ulp relative change of every input coordinate
        x = x * (1 + np.random.default_rng(perturb).choice([-1.0, 1.0], x.shape) * 2.0**-52)
    gp = R.gp_init([R.cf(p["kind"], lscale=p["lscale"], magn=p["magn"])], R.lik("gaussian", sigma=p["sigma"]))
    with np.errstate(invalid="ignore"):
        gp = R.gp_fit(gp, x, p["y"])
        pr = R.gp_pred(gp, p["xt"], var=True)
        lo = R.gp_loo(gp, x, p["y"], quad_order=quad_order)
    return gp.fit["log_evidence"], pr, lo["loos"]


def relmax(a, b):
    """Max-norm relative difference over the entries where the oracle is finite.

    The reference's LOO variance 1 / (1 / post_var - 1 / V) has no guard: for tiny
    sigma post_var can round to <= 0 and the oracle returns NaN densities there
    (sqrt of a negative variance); the sign of such a rounding-level quantity is not
    a property of the algorithm, so those entries are not compared."""
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    ok = np.isfinite(b)
    if not ok.any():
        return 0.0
    return float(np.max(np.abs(a[ok] - b[ok])) / max(np.max(np.abs(b[ok])), 1e-300))


def lml_err(a, b, n):
    """|a - b| relative to max(|b|, n): the evidence is a sum of n-extensive terms
    (n/2 log 2 pi alone), so a near-zero evidence would turn rounding-level absolute
    differences into large relative ones."""
    return abs(a - b) / max(abs(b), n)


# Unit roundoff of the contraction: 2^-53 on the FP64 pipe, 2^-41 for the
# 5-slice BF16 products of the mixed plan.
AMPLIFY = {"fp64": 1.0, "mixed": 2.0**12}


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batched_matches_oracle(precision):
    """Evidence within 1e-10 (FP64) / 1e-8 (mixed) of max(|LML|, n). Predictions and LOO
    densities within max(base, 100 x sensitivity x roundoff ratio), where the
    sensitivity is the oracle's own max-norm change under a one-ulp change of x: the
    LOO variance of small-sigma problems cancels (D - D^2 binv / V), so a fixed bound
    would test the conditioning of the problem, not the kernels."""
    probs = make_problems(48, seed=5)
    res = gp_fit_batched(probs, precision=precision)
    tol_l, tol_v = (1e-10, 1e-9) if precision == "fp64" else (1e-8, 1e-6)
    bad = []
    for i, (p, r) in enumerate(zip(probs, res)):
        n = len(p["y"])
        lml, pr, loos = oracle_solve(p)
        _, pr2, loos2 = oracle_solve(p, perturb=i)
        amp = 100 * AMPLIFY[precision]
        checks = [
            ("lml", lml_err(r["log_evidence"], lml, n), tol_l),
            ("mean", relmax(r["mean"], pr["mean"]), max(tol_v, amp * relmax(pr2["mean"], pr["mean"]))),
            ("var", relmax(r["var"], pr["var"]), max(10 * tol_v, amp * relmax(pr2["var"], pr["var"]))),
            ("loos", relmax(r["loos"], loos), max(tol_v, amp * relmax(loos2, loos))),
        ]
        for name, err, tol in checks:
            if not err <= tol:
                bad.append((i, n, p["kind"], round(p["sigma"], 4), name, err, tol))
    assert not bad, bad


def test_batched_rerun_and_upload_are_consistent():
    probs = make_problems(20, seed=9, nmax=200)
    plan = BatchPlan(probs, precision="mixed")
    plan.run()
    a = plan.results()
    plan.run()
    b = plan.results()
    for u, v in zip(a, b):
        assert u["log_evidence"] == v["log_evidence"]  # deterministic replay
    probs2 = make_problems(20, seed=9, nmax=200)
    for p in probs2:
        p["y"] = p["y"] + 0.5
    plan.upload(probs2)
    plan.run()
    c = plan.results()
    lml, _, _ = oracle_solve(probs2[3])
    assert lml_err(c[3]["log_evidence"], lml, len(probs2[3]["y"])) <= 1e-8
    info = plan.info()
    assert sum(cnt for _, cnt, _ in info["buckets"]) == 20
    plan.close()
