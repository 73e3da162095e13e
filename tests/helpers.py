"""Shared test helpers: matched product / oracle models on the same inputs."""
import copy

import numpy as np

import gplite_gb300 as G
from oracle import gplite_ref as R


def cf_zoo():
    """The seven covariance functions of tests/testthat/test_basic.R:15-23."""
    return [G.cf_const(), G.cf_lin(), G.cf_sexp(), G.cf_matern32(), G.cf_matern52(), G.cf_nn(),
            G.cf_periodic()]


def basic_models():
    """All cfs alone, all pairs, all triple products (test_basic.R:30-58)."""
    import itertools
    import warnings
    zoo = cf_zoo()
    out = [[c] for c in zoo]
    out += [[a, b] for a, b in itertools.combinations(zoo, 2)]
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        out += [[a * b * c] for a, b, c in itertools.combinations(zoo, 3)]
    return out


def oracle_gp(gp):
    return R.gp_init(copy.deepcopy(gp.cfs), copy.deepcopy(gp.lik), copy.deepcopy(gp.method),
                     copy.deepcopy(gp.approx))


def rel_err(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300)))


def close(a, b, rtol, atol=0.0):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return bool(np.all(np.abs(a - b) <= atol + rtol * np.abs(b)))
