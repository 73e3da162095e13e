"""Request server (gpgp_server_*): results alone equal results in the mix,
resident models, HBM-budget admission, and parity of served fits with the
oracle's gp_fit / gp_pred."""
import numpy as np
import pytest

import gplite_gb300 as G
from gplite_gb300 import _lib as L
from gplite_gb300.server import GPServer
from oracle import gplite_ref as R

pytestmark = pytest.mark.gpu


def make_requests(seed=3):
    """Mixed sizes and kinds: batch-lane Gaussians (n <= 1024), large Gaussians,
    Poisson under Laplace, a compound kernel and a FITC fit (worker lanes)."""
    rng = np.random.default_rng(seed)
    reqs = []
    for i in range(28):
        n = int(np.exp(rng.uniform(np.log(32), np.log(1800))))
        x = rng.uniform(-2, 2, (n, 2))
        f = np.sin(2 * x[:, 0]) * np.cos(x[:, 1])
        xt = rng.uniform(-2, 2, (int(rng.integers(1, 64)), 2))
        ls = float(np.exp(rng.uniform(np.log(0.3), np.log(1.5))))
        if i % 5 == 4:
            y = rng.poisson(np.exp(f)).astype(float)
            gp = G.gp_init(G.cf_sexp(lscale=ls, magn=1.0), G.lik_poisson())
        elif i % 7 == 6:
            y = f + 0.1 * rng.standard_normal(n)
            gp = G.gp_init([G.cf_sexp(lscale=ls, magn=1.0), G.cf_const(magn=0.5)], G.lik_gaussian(sigma=0.1))
        else:
            sig = float(rng.uniform(0.05, 0.3))
            y = f + sig * rng.standard_normal(n)
            gp = G.gp_init(G.cf_sexp(lscale=ls, magn=1.0), G.lik_gaussian(sigma=sig))
        reqs.append((gp, x, y, xt))
    n = 3000
    x = rng.uniform(-2, 2, (n, 2))
    y = np.sin(2 * x[:, 0]) + 0.1 * rng.standard_normal(n)
    z = x[rng.choice(n, 48, replace=False)]
    gp = G.gp_init(G.cf_sexp(lscale=0.8, magn=1.0), G.lik_gaussian(sigma=0.1), method=G.method_fitc(inducing=z))
    reqs.append((gp, x, y, rng.uniform(-2, 2, (40, 2))))
    return reqs


def serve(server, reqs, together):
    out = []
    if together:
        tickets = [server.submit(gp, x, y, xt) for gp, x, y, xt in reqs]
        for t in tickets:
            out.append(server.poll(t, wait_ms=-1))
    else:
        for gp, x, y, xt in reqs:
            out.append(server.poll(server.submit(gp, x, y, xt), wait_ms=-1))
    return out


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_alone_equals_mix(precision):
    """Each request's evidence, mean and variance are the same (bit for bit) when it
    is served alone and when it is served among all the others."""
    reqs = make_requests()
    with GPServer(precision=precision, workers=4) as s:
        alone = serve(s, reqs, together=False)
        mix = serve(s, reqs, together=True)
        st = s.stats()
    lanes = set()
    for a, b in zip(alone, mix):
        assert a["status"] == 0 and b["status"] == 0
        assert a["log_evidence"] == b["log_evidence"]
        np.testing.assert_array_equal(a["mean"], b["mean"])
        np.testing.assert_array_equal(a["var"], b["var"])
        lanes.add(a["lane"])
    assert lanes == {"batch", "worker"}
    assert st["completed"] == 2 * len(reqs) and st["failed"] == 0
    assert st["batches"] < st["batched_requests"]  # the mix was batched
    assert st["bytes_peak"] <= st["budget"]


def test_served_fits_match_oracle():
    """Served FP64 results against the oracle's gp_fit / gp_pred (1e-10 relative on the
    evidence, 1e-9 of the largest entry on mean and variance)."""
    reqs = [r for r in make_requests(seed=8)[:12]]
    with GPServer(precision="fp64") as s:
        res = serve(s, reqs, together=True)
    for (gp, x, y, xt), r in zip(reqs, res):
        cfs = []
        for c in gp.cfs:
            if c.kind == "const":
                cfs.append(R.cf("const", magn=c.magn))
            else:
                cfs.append(R.cf(c.kind, lscale=c.lscale, magn=c.magn))
        lk = R.lik("gaussian", sigma=gp.lik.sigma) if gp.lik.kind == "gaussian" else R.lik("poisson")
        og = R.gp_fit(R.gp_init(cfs, lk), x, y)
        po = R.gp_pred(og, xt, var=True)
        lml = og.fit["log_evidence"]
        assert abs(r["log_evidence"] - lml) <= 1e-10 * max(abs(lml), len(y))
        assert np.max(np.abs(r["mean"] - po["mean"])) <= 1e-9 * np.max(np.abs(po["mean"]))
        assert np.max(np.abs(r["var"] - po["var"])) <= 1e-9 * np.max(np.abs(po["var"]))


def test_resident_model_predictions():
    """keep = 1 leaves the factor on the device: later predictions equal gp_pred on a
    model fitted directly; after release the model id is refused."""
    rng = np.random.default_rng(4)
    n = 1500
    x = rng.uniform(-2, 2, (n, 2))
    y = np.sin(3 * x[:, 0]) + 0.1 * rng.standard_normal(n)
    gp = G.gp_init(G.cf_matern52(lscale=0.6, magn=1.0), G.lik_gaussian(sigma=0.1))
    xt1, xt2 = rng.uniform(-2, 2, (100, 2)), rng.uniform(-2, 2, (333, 2))
    with GPServer(precision="fp64", workers=2) as s:
        r = s.poll(s.submit(gp, x, y, xt1, keep=True))
        assert r["status"] == 0 and r["model"] >= 0
        st = s.stats()
        assert st["bytes_resident"] > 0
        p = s.poll(s.submit_pred(r["model"], xt2))
        s.release(r["model"])
        with pytest.raises(L.GpgpError):
            s.submit_pred(r["model"], xt2)
        assert s.stats()["bytes_resident"] == 0
    ref = G.gp_fit(G.gp_init(G.cf_matern52(lscale=0.6, magn=1.0), G.lik_gaussian(sigma=0.1)), x, y)
    q = G.gp_pred(ref, xt2, var=True)
    assert abs(r["log_evidence"] - ref.fit["log_evidence"]) <= 1e-12 * abs(ref.fit["log_evidence"])
    np.testing.assert_allclose(p["mean"], q["mean"], rtol=0, atol=1e-12 * np.max(np.abs(q["mean"])))
    np.testing.assert_allclose(p["var"], q["var"], rtol=0, atol=1e-12 * np.max(np.abs(q["var"])))


def test_budget_admission():
    """A request larger than the whole budget fails with out-of-memory; under a budget
    that holds only a few requests at a time, all complete and the peak stays below it."""
    rng = np.random.default_rng(6)
    big_n = 6000
    x = rng.uniform(-2, 2, (big_n, 2))
    y = np.sin(x[:, 0]) + 0.1 * rng.standard_normal(big_n)
    gp = G.gp_init(G.cf_sexp(lscale=0.5), G.lik_gaussian(sigma=0.1))
    budget = 200 << 20
    with GPServer(precision="fp64", workers=3, hbm_budget=budget) as s:
        r = s.poll(s.submit(gp, x, y, x[:10]))
        assert r["status"] == L.EOOM
        tickets = []
        for i in range(16):
            n = 1200 + 50 * i
            xi = rng.uniform(-2, 2, (n, 2))
            yi = np.sin(xi[:, 0]) + 0.1 * rng.standard_normal(n)
            gpi = G.gp_init([G.cf_sexp(lscale=0.5), G.cf_const(magn=0.3)], G.lik_gaussian(sigma=0.1))
            tickets.append(s.submit(gpi, xi, yi, xi[:20]))
        for t in tickets:
            assert s.poll(t)["status"] == 0
        st = s.stats()
    assert st["bytes_peak"] <= budget
    assert st["failed"] == 1
