"""Failure detection without a GPU fault: a bounded device wait that runs out
returns GPGP_ETIMEOUT and leaves the context usable; NaN/Inf inputs are refused
with GPGP_ENAN; a non-positive-definite factor gives GPGP_ENOT_PD and -Inf; in
the server a bad request fails alone."""
import numpy as np
import pytest

import gplite_gb300 as G
from gplite_gb300 import _lib as L
from gplite_gb300.server import GPServer

pytestmark = pytest.mark.gpu


def _data(n=120, seed=0):
    rng = np.random.default_rng(seed)
    x = rng.uniform(-2, 2, (n, 2))
    return x, np.sin(x[:, 0]) + 0.1 * rng.standard_normal(n)


def test_bounded_wait_times_out_and_context_survives():
    ctx = L.default_context(0)
    st = L.load().gpgp_wait_selftest(ctx.h, 2000)
    assert st == L.ETIMEOUT
    x, y = _data()
    gp = G.gp_fit(G.gp_init(G.cf_sexp(lscale=0.5), G.lik_gaussian(sigma=0.1)), x, y)
    assert np.isfinite(gp.fit["log_evidence"])


@pytest.mark.parametrize("where", ["x", "y"])
@pytest.mark.parametrize("bad", [np.nan, np.inf])
def test_nonfinite_inputs_are_refused(where, bad):
    x, y = _data()
    x, y = x.copy(), y.copy()
    if where == "x":
        x[7, 1] = bad
    else:
        y[3] = bad
    with pytest.raises(L.GpgpError) as e:
        G.gp_fit(G.gp_init(G.cf_sexp(lscale=0.5), G.lik_gaussian(sigma=0.1)), x, y)
    assert e.value.status == L.ENAN


def test_not_positive_definite_and_server_isolation():
    """A negative jitter makes B indefinite: the factorisation reports the failing pivot;
    in the server a request with NaN data fails and the others do not."""
    x, y = _data(64)
    gp = G.gp_init(G.cf_sexp(lscale=0.5), G.lik_gaussian(sigma=0.01))
    with pytest.raises(L.NotPositiveDefinite):
        G.gp_fit(gp, x, y, jitter=-10.0)
    xb, yb = _data(80, seed=3)
    yb = yb.copy()
    yb[5] = np.nan
    good = [_data(90 + 10 * i, seed=10 + i) for i in range(4)]
    with GPServer(precision="fp64", workers=2) as s:
        tb = s.submit(G.gp_init(G.cf_sexp(lscale=0.5), G.lik_gaussian(sigma=0.1)), xb, yb, xb[:5])
        tg = [s.submit(G.gp_init([G.cf_sexp(lscale=0.5), G.cf_const(magn=0.2)], G.lik_gaussian(sigma=0.1)),
                       xg, yg, xg[:5]) for xg, yg in good]
        rb = s.poll(tb)
        rg = [s.poll(t) for t in tg]
    assert rb["status"] != 0
    assert all(r["status"] == 0 and np.isfinite(r["log_evidence"]) for r in rg)
