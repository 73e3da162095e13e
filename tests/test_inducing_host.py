"""Host logic of the inducing-input selection (get_inducing and bin,
R/gp_fit.R:192-259), with the device k-means replaced by a stub that returns
its initial centres: binning, per-bin counts, scaling and the given-inputs path."""
import numpy as np

import gplite_gb300 as G
from gplite_gb300 import gp as GP


def _stub(monkeypatch, calls):
    def fake(x, k, init, max_iter=10, device=0):
        calls.append((np.array(x), k))
        return np.array(init), 1, 0.0

    monkeypatch.setattr(GP, "kmeans", fake)


def test_bin_follows_reference_cutpoints():
    x = np.column_stack([np.arange(10.0), np.zeros(10)])
    bins = GP._bin(x, 3, 0)
    # cutpoints seq(min - 2 eps, max + 2 eps, len = 4) = (-4.4e-16, 3 - 4.4e-16, 6, 9) with
    # strict inequalities: 6 lies on a cutpoint and 9 on the upper end (9 + 2 eps rounds to 9),
    # so both fall in no bin, as in the reference
    assert [b[:, 0].tolist() for b in bins] == [[0, 1, 2], [3, 4, 5], [7, 8]]
    y = np.column_stack([[0.0, 1.0, 2.5, 4.0, 5.5, 7.0, 1.0 - 1e-9, 1e-3], np.ones(8)])
    assert [len(b) for b in GP._bin(y, 2, 0)] == [5, 2]  # cut at 3.5; the maximum 7 again in none


def test_binned_inducing_counts_and_order(monkeypatch):
    calls = []
    _stub(monkeypatch, calls)
    rng = np.random.default_rng(0)
    x = np.column_stack([np.r_[rng.uniform(0, 1, 50), rng.uniform(1, 2, 200), rng.uniform(2, 3, 100)],
                         rng.standard_normal(350)])
    gp = G.gp_init(G.cf_sexp(), method=G.method_fitc(num_inducing=11, bin_along=0, bin_count=3))
    z = GP.get_inducing(gp, x)
    assert z.shape == (11, 2)
    # the largest bin first; the leftover 11 - 3*3 = 2 go to the two largest bins
    assert [k for _, k in calls] == [4, 4, 3]
    assert [len(c[0]) for c in calls] == [200, 100, 50]
    # the stub returns scaled data rows, so the unscaled centres are rows of x in each bin
    for row in z:
        assert np.min(np.max(np.abs(x - row), axis=1)) < 1e-12


def test_unbinned_inducing_is_scaled(monkeypatch):
    calls = []
    _stub(monkeypatch, calls)
    rng = np.random.default_rng(1)
    x = rng.normal(5.0, 3.0, (500, 3))
    gp = G.gp_init(G.cf_sexp(), method=G.method_fitc(num_inducing=20))
    z = GP.get_inducing(gp, x)
    xs, k = calls[0]
    assert k == 20 and xs.shape == (500, 3)
    assert np.allclose(xs.mean(0), 0.0, atol=1e-12) and np.allclose(xs.std(0, ddof=1), 1.0)
    assert z.shape == (20, 3)
    # the same seed gives the same selection
    calls.clear()
    assert np.array_equal(GP.get_inducing(gp, x), z)


def test_given_inducing_inputs_are_kept(monkeypatch):
    calls = []
    _stub(monkeypatch, calls)
    zin = np.linspace(0, 1, 8)[:, None]
    gp = G.gp_init(G.cf_sexp(), method=G.method_fitc(inducing=zin))
    assert GP.get_inducing(gp, np.zeros((30, 1))) is gp.method.inducing
    assert calls == []
