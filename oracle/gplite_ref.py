"""FP64 NumPy/SciPy restatement of gplite's GP hot path (TEST INFRASTRUCTURE ONLY).

Every function restates one reference function, named in its docstring by
file:line of the R package gplite 0.13.0 (paths relative to the package root).
Matrices follow R's conventions: inputs are n-by-d, column-major semantics are
irrelevant here because NumPy holds the values; ``chol`` is R's upper factor,
``t(chol(B))`` the lower one. Formula order follows the reference (B
factorisation, log-evidence expression), not textbook shortcuts, so that the
CUDA library can be held to 1e-10 against it.

Objects are duck-typed: a covariance function is any object with attributes
``kind`` ('const', 'lin', 'sexp', 'matern32', 'matern52', 'nn', 'periodic',
'prod'), ``vars`` (None or 0-based column indices), ``normalize``, ``means``,
``scales``, ``priors`` (dict name -> prior) and its parameters by name
(``lscale``, ``magn``, ``sigma0``, ``sigma``, ``period``); ``base`` for
periodic, ``cfs`` for products. A likelihood has ``kind`` ('gaussian',
'bernoulli', 'binomial', 'betabinom', 'poisson'), ``link`` and its parameters.
The constructors at the bottom build such objects without the product package.

Parity: see the package docstring (pinned to the reference's closed-form
known-answer tests; Laplace/EP/FITC values partially unpinned).
"""
from __future__ import annotations

import math
import warnings
from types import SimpleNamespace

import numpy as np
from scipy import linalg as sla
from scipy import special as sps

# ----------------------------------------------------------------------------
# parameters (R/cf.R:283-396, R/lik.R:118-168, R/gp.R:149-165, R/misc.R:33-56)
# ----------------------------------------------------------------------------

PARAM_NAMES = {
    "const": ["magn"],
    "lin": ["magn"],
    "sexp": ["lscale", "magn"],
    "matern32": ["lscale", "magn"],
    "matern52": ["lscale", "magn"],
    "nn": ["sigma0", "sigma", "magn"],
    "periodic": ["period"],
    "gaussian": ["sigma"],
    "bernoulli": [],
    "binomial": [],
    "betabinom": ["phi"],
    "poisson": [],
}


def _is_fixed(obj, name):
    """is_fixed (R/misc.R:33-39)."""
    pr = getattr(obj, "priors", {}) or {}
    p = pr.get(name)
    return p is not None and p.kind == "fixed"


def _obj_name(obj, is_lik=False):
    return ("lik_" if is_lik else "cf_") + obj.kind


def get_param_cf(cf):
    """get_param.cf / .cf_periodic / .cf_prod (R/cf.R:313-344)."""
    if cf.kind == "prod":
        names, vals = [], []
        for c in cf.cfs:
            n_, v_ = get_param_cf(c)
            names += n_
            vals += v_
        return names, vals
    if cf.kind == "periodic":
        n_, v_ = get_param_cf(cf.base)
        n_ = ["cf_periodic." + s.split(".", 1)[1] for s in n_]
        if not _is_fixed(cf, "period"):
            n_ = ["cf_periodic.period"] + n_
            v_ = [math.log(cf.period)] + v_
        return n_, v_
    names, vals = [], []
    for nm in PARAM_NAMES[cf.kind]:
        if _is_fixed(cf, nm):
            continue
        names.append(_obj_name(cf) + "." + nm)
        vals.append(math.log(getattr(cf, nm)))
    return names, vals


def get_param_lik(lik):
    """get_param.lik (R/lik.R:146-155)."""
    names, vals = [], []
    for nm in PARAM_NAMES[lik.kind]:
        if _is_fixed(lik, nm):
            continue
        names.append(_obj_name(lik, True) + "." + nm)
        vals.append(math.log(getattr(lik, nm)))
    return names, vals


def get_param(gp):
    """get_param.gp (R/gp.R:149-155): cfs in declared order, then likelihood."""
    names, vals = [], []
    for cf in gp.cfs:
        n_, v_ = get_param_cf(cf)
        names += n_
        vals += v_
    n_, v_ = get_param_lik(gp.lik)
    return names + n_, np.array(vals + v_, dtype=np.float64)


def _set_param_cf(cf, vals, exp=math.exp):
    """set_param.cf / .cf_periodic / .cf_prod (R/cf.R:348-396). Returns #consumed.
    (exp = np.exp lets the complex-step derivative check set complex values.)"""
    if cf.kind == "prod":
        j = 0
        for c in cf.cfs:
            j += _set_param_cf(c, vals[j:], exp)
        return j
    if cf.kind == "periodic":
        j = 0
        if not _is_fixed(cf, "period"):
            cf.period = exp(vals[0])
            j = 1
        return j + _set_param_cf(cf.base, vals[j:], exp)
    j = 0
    for nm in PARAM_NAMES[cf.kind]:
        if _is_fixed(cf, nm):
            continue
        setattr(cf, nm, exp(vals[j]))
        j += 1
    return j


def set_param(gp, vals):
    """set_param.gp (R/gp.R:158-165); marks the model as not fitted."""
    vals = list(np.asarray(vals, dtype=np.float64))
    j = 0
    for cf in gp.cfs:
        j += _set_param_cf(cf, vals[j:])
    for nm in PARAM_NAMES[gp.lik.kind]:
        if _is_fixed(gp.lik, nm):
            continue
        setattr(gp.lik, nm, math.exp(vals[j]))
        j += 1
    gp.fitted = False
    return gp


# ----------------------------------------------------------------------------
# priors (R/priors.R:96-112)
# ----------------------------------------------------------------------------

def lpdf_prior_one(prior, param):
    """lpdf_prior.prior_* (R/priors.R:96-112)."""
    if prior is None or prior.kind in ("fixed", "logunif"):
        return 0.0
    if prior.kind == "half_t":
        theta = math.exp(param)
        df, sc = prior.df, prior.scale
        t = theta / sc
        # stats::dt(t, df, log=TRUE)
        ldt = (sps.gammaln((df + 1) / 2) - sps.gammaln(df / 2) - 0.5 * math.log(df * math.pi)
               - (df + 1) / 2 * math.log1p(t * t / df))
        return math.log(2) - math.log(sc) + ldt + param
    if prior.kind == "lognormal":
        return -0.5 * math.log(2 * math.pi) - math.log(prior.scale) - 0.5 * ((param - prior.loc) / prior.scale) ** 2
    raise ValueError(prior.kind)


def _lpdf_prior_cf(cf):
    """lpdf_prior.cf / .cf_prod / .cf_periodic (R/cf.R:503-528)."""
    if cf.kind == "prod":
        return sum(_lpdf_prior_cf(c) for c in cf.cfs)
    if cf.kind == "periodic":
        lp = 0.0
        if not _is_fixed(cf, "period"):
            lp += lpdf_prior_one(cf.priors.get("period"), math.log(cf.period))
        return lp + _lpdf_prior_cf(cf.base)
    lp = 0.0
    for nm in PARAM_NAMES[cf.kind]:
        if _is_fixed(cf, nm):
            continue
        lp += lpdf_prior_one(cf.priors.get(nm), math.log(getattr(cf, nm)))
    return lp


def lpdf_prior(gp):
    """lpdf_prior.gp (R/gp.R:167-169)."""
    lp = sum(_lpdf_prior_cf(cf) for cf in gp.cfs)
    for nm in PARAM_NAMES[gp.lik.kind]:
        if not _is_fixed(gp.lik, nm):
            lp += lpdf_prior_one(gp.lik.priors.get(nm), math.log(getattr(gp.lik, nm)))
    return lp


# ----------------------------------------------------------------------------
# inputs and covariance functions (R/misc.R:17-31, R/cf.R:402-497, src/cf.cpp)
# ----------------------------------------------------------------------------

def as_matrix(x):
    x = np.asarray(x)
    if not np.iscomplexobj(x):  # complex only in the complex-step derivative check
        x = x.astype(np.float64, copy=False)
    return x.reshape(-1, 1) if x.ndim == 1 else x


def prepare_inputmat(cf, x):
    """prepare_inputmat (R/misc.R:17-31): column subset, then (x - mean) / scale."""
    x = as_matrix(x)
    if cf.vars is not None:
        x = x[:, list(cf.vars)]
    if getattr(cf, "normalize", False) and getattr(cf, "means", None) is not None \
            and getattr(cf, "scales", None) is not None:
        x = (x - np.asarray(cf.means)) / np.asarray(cf.scales)
    return x


def learn_scales(cfs, x):
    """learn_scales.cf / .cf_prod / .cf_periodic (R/cf.R:824-855): colMeans, sd (n-1)."""
    x = as_matrix(x)
    for cf in cfs:
        if cf.kind == "prod":
            learn_scales(cf.cfs, x)
        elif cf.kind == "periodic":
            continue
        else:
            xs = x if cf.vars is None else x[:, list(cf.vars)]
            cf.means = xs.mean(axis=0)
            cf.scales = xs.std(axis=0, ddof=1)


def _sqdist(x1, x2):
    # sum(square(x1.row(i) - x2.row(j))) accumulated over columns in order (src/cf.cpp:37)
    # (complex inputs only arise in the complex-step derivative check of the gradient)
    r2 = np.zeros((x1.shape[0], x2.shape[0]), dtype=np.result_type(x1, x2, np.float64))
    for k in range(x1.shape[1]):
        diff = x1[:, k][:, None] - x2[:, k][None, :]
        r2 += diff * diff
    return r2


def _sqdist_diag(x1, x2):
    n = min(x1.shape[0], x2.shape[0])
    r2 = np.zeros(n, dtype=np.result_type(x1, x2, np.float64))
    for k in range(x1.shape[1]):
        diff = x1[:n, k] - x2[:n, k]
        r2 += diff * diff
    return r2


def cf_sexp_c(x1, x2, lscale, magn, diag_only=False):
    """cf_sexp_c (src/cf.cpp:9-42)."""
    r2 = _sqdist_diag(x1, x2) if diag_only else _sqdist(x1, x2)
    return magn * magn * np.exp(-0.5 * r2 / (lscale * lscale))


def cf_matern32_c(x1, x2, lscale, magn, diag_only=False):
    """cf_matern32_c (src/cf.cpp:48-80)."""
    r = np.sqrt(_sqdist_diag(x1, x2) if diag_only else _sqdist(x1, x2))
    return magn * magn * (1.0 + math.sqrt(3.0) * r / lscale) * np.exp(-math.sqrt(3.0) * r / lscale)


def cf_matern52_c(x1, x2, lscale, magn, diag_only=False):
    """cf_matern52_c (src/cf.cpp:86-119)."""
    r = np.sqrt(_sqdist_diag(x1, x2) if diag_only else _sqdist(x1, x2))
    return magn * magn * (1.0 + math.sqrt(5.0) * r / lscale + 5.0 * r * r / (3.0 * lscale * lscale)) \
        * np.exp(-math.sqrt(5.0) * r / lscale)


def cf_nn_c(x1, x2, sigma0, sigma, magn, diag_only=False):
    """cf_nn_c (src/cf.cpp:125-162)."""
    s0 = sigma0 * sigma0 * sigma * sigma
    a1 = x1 * sigma
    a2 = x2 * sigma
    if diag_only:
        n = min(a1.shape[0], a2.shape[0])
        a1, a2 = a1[:n], a2[:n]
        a = s0 + (a1 * a2).sum(1)
        b = s0 + (a1 * a1).sum(1)
        c = s0 + (a2 * a2).sum(1)
    else:
        a = s0 + a1 @ a2.T
        b = (s0 + (a1 * a1).sum(1))[:, None]
        c = (s0 + (a2 * a2).sum(1))[None, :]
    return magn * magn * (2.0 / math.pi) * np.arcsin(2 * a / np.sqrt((1 + 2 * b) * (1 + 2 * c)))


def eval_cf_one(cf, x1, x2, diag_only=False):
    """eval_cf.cf_* (R/cf.R:413-497)."""
    if cf.kind == "prod":
        K = 1.0
        for c in cf.cfs:
            K = K * eval_cf_one(c, x1, x2, diag_only)
        return K
    x1 = prepare_inputmat(cf, x1)
    x2 = prepare_inputmat(cf, x2)
    n1, n2 = x1.shape[0], x2.shape[0]
    if cf.kind == "const":
        if diag_only:
            return np.full(min(n1, n2), cf.magn ** 2)
        return np.full((n1, n2), cf.magn ** 2)
    if cf.kind == "lin":
        K = cf.magn ** 2 * (x1 @ x2.T)
        return np.diag(K).copy() if diag_only else K
    if cf.kind == "sexp":
        return cf_sexp_c(x1, x2, cf.lscale, cf.magn, diag_only)
    if cf.kind == "matern32":
        return cf_matern32_c(x1, x2, cf.lscale, cf.magn, diag_only)
    if cf.kind == "matern52":
        return cf_matern52_c(x1, x2, cf.lscale, cf.magn, diag_only)
    if cf.kind == "nn":
        return cf_nn_c(x1, x2, cf.sigma0, cf.sigma, cf.magn, diag_only)
    if cf.kind == "periodic":
        w = 2 * math.pi / cf.period
        t1 = np.hstack([np.sin(w * x1), np.cos(w * x1)])
        t2 = np.hstack([np.sin(w * x2), np.cos(w * x2)])
        return eval_cf_one(cf.base, t1, t2, diag_only)
    raise ValueError(cf.kind)


def eval_cf(cfs, x1, x2, cfind=None, diag_only=False, threads=1):
    """eval_cf.list (R/cf.R:402-411): sum over the selected covariance functions.
    threads > 1 evaluates row blocks of x1 in parallel threads (every covariance
    function is row-separable, so the values are the same)."""
    idx = range(len(cfs)) if cfind is None else cfind
    x1 = as_matrix(x1)
    if threads > 1 and not diag_only and x1.shape[0] >= 4 * 256:
        from concurrent.futures import ThreadPoolExecutor
        bounds = np.linspace(0, x1.shape[0], 4 * threads + 1).astype(int)
        with ThreadPoolExecutor(threads) as ex:
            parts = list(ex.map(lambda b: eval_cf(cfs, x1[b[0]:b[1]], x2, cfind),
                                zip(bounds[:-1], bounds[1:])))
        return np.vstack([np.broadcast_to(p, (b1 - b0, as_matrix(x2).shape[0]))
                          for p, b0, b1 in zip(parts, bounds[:-1], bounds[1:])])
    K = 0.0
    for k in idx:
        K = K + eval_cf_one(cfs[k], x1, x2, diag_only)
    return K


# ----------------------------------------------------------------------------
# likelihoods (R/lik.R:188-498)
# ----------------------------------------------------------------------------

def add_offset(f, offset):
    """add_offset (R/misc.R:6-15)."""
    return f if offset is None else f + offset


def get_response(lik, f):
    """get_response.lik_* (R/lik.R:460-498)."""
    if lik.kind == "gaussian":
        return f
    if lik.kind in ("bernoulli", "binomial", "betabinom"):
        if lik.link == "probit":
            return sps.ndtr(f)
        if lik.link == "logit":
            return 1 / (1 + np.exp(-f))
        raise ValueError(lik.link)
    if lik.kind == "poisson":
        return np.exp(f)
    raise ValueError(lik.kind)


def _xlogy(x, y):
    with np.errstate(divide="ignore", invalid="ignore"):
        out = x * np.log(y)
    return np.where(x == 0, 0.0, out)


def get_loglik(lik, f, y, trials=None, offset=None, sum_=True):
    """get_loglik.lik_* (R/lik.R:301-366). dbinom/dpois/dnorm by closed form (R nmath agrees
    to rounding away from the extreme tails)."""
    f = np.asarray(f, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    if f.ndim == 2:  # an n-by-q quadrature grid: per-observation quantities broadcast along rows
        y = y[:, None]
        if trials is not None:
            trials = np.asarray(trials, dtype=np.float64)[:, None]
        if offset is not None:
            offset = np.asarray(offset, dtype=np.float64)[:, None]
    f = add_offset(f, offset)
    if lik.kind == "gaussian":
        s = lik.sigma
        ll = -math.log(s) - 0.5 * math.log(2 * math.pi) - 0.5 * ((y - f) / s) ** 2
    elif lik.kind in ("bernoulli", "binomial"):
        N = np.ones_like(y) if lik.kind == "bernoulli" else np.asarray(trials, dtype=np.float64)
        mu = get_response(lik, f)
        lch = sps.gammaln(N + 1) - sps.gammaln(y + 1) - sps.gammaln(N - y + 1)
        ll = lch + _xlogy(y, mu) + _xlogy(N - y, 1 - mu)
    elif lik.kind == "poisson":
        mu = get_response(lik, f)
        ll = _xlogy(y, mu) - mu - sps.gammaln(y + 1)
    elif lik.kind == "betabinom":
        N = np.asarray(trials, dtype=np.float64)
        mu = get_response(lik, f)
        a = mu / lik.phi
        b = (1 - mu) / lik.phi
        g = sps.gammaln
        term1 = g(N + 1) - g(y + 1) - g(N - y + 1)
        term2 = g(y + a) + g(N - y + b) - g(N + a + b)
        term3 = g(a + b) - g(a) - g(b)
        ll = term1 + term2 + term3  # R/lik.R:344-347
    else:
        raise ValueError(lik.kind)
    ll = np.broadcast_to(ll, f.shape).astype(np.float64)
    return float(ll.sum()) if sum_ else ll


def get_loglik_d(lik, f, y, trials=None, offset=None):
    """get_loglik_d.lik_* (R/lik.R:372-443)."""
    f = add_offset(np.asarray(f, dtype=np.float64), offset)
    y = np.asarray(y, dtype=np.float64)
    mu = get_response(lik, f)
    if lik.kind in ("bernoulli", "binomial"):
        N = np.ones_like(y) if lik.kind == "bernoulli" else np.asarray(trials, dtype=np.float64)
        dmu = np.exp(-0.5 * f * f) / math.sqrt(2 * math.pi) if lik.link == "probit" else mu * (1 - mu)
        return dmu * (y / mu - (N - y) / (1 - mu))
    if lik.kind == "poisson":
        return (y / mu - 1) * mu
    if lik.kind == "betabinom":
        N = np.asarray(trials, dtype=np.float64)
        phi = lik.phi
        a = mu / phi
        b = (1 - mu) / phi
        dmu = np.exp(-0.5 * f * f) / math.sqrt(2 * math.pi) if lik.link == "probit" else mu * (1 - mu)
        dg = sps.digamma
        return (dmu / phi) * (dg(y + a) - dg(N - y + b)) + (dmu / phi) * (-dg(a) + dg(b))
    raise ValueError(lik.kind)


def get_loglik_d2(lik, f, y, trials=None, offset=None, eps=1e-6):
    """get_loglik_d2.lik (R/lik.R:449-454): forward finite difference of the gradient."""
    g = get_loglik_d(lik, f, y, trials, offset)
    ge = get_loglik_d(lik, f + eps, y, trials, offset)
    return g, (ge - g) / eps


def get_pseudodata_la(lik, f, y, trials=None, offset=None, min_abs_curvature=1e-12):
    """get_pseudodata_la.lik_gaussian / .lik (R/lik.R:188-201)."""
    n = len(y)
    if lik.kind == "gaussian":
        return np.asarray(y, dtype=np.float64).copy(), lik.sigma ** 2 * np.ones(n)
    f = np.asarray(f, dtype=np.float64).ravel()
    g, g2 = get_loglik_d2(lik, f, y, trials, offset)
    g2 = np.sign(g2) * np.maximum(np.abs(g2), min_abs_curvature)
    with np.errstate(divide="ignore", invalid="ignore"):
        return f - g / g2, -1 / g2


# ----------------------------------------------------------------------------
# Gauss-Hermite quadrature (R/quadrature.R:1-44), logsumexp (R/gp_loo.R:136-144)
# ----------------------------------------------------------------------------

def hermite_polynomials(n):
    """hermite_polynomials (R/quadrature.R:1-16): probabilists' He_k coefficients, row k."""
    c = np.zeros((n + 1, n + 1))
    c[0, 0] = 1
    if n == 0:
        return c
    c[1, 1] = 1
    for i in range(2, n + 1):
        c[i, :] = np.concatenate([[0.0], c[i - 1, :n]]) - (i - 1) * c[i - 2, :]
    return c


def gauss_hermite_points(p):
    """gauss_hermite_points (R/quadrature.R:28-34): nodes = real roots of He_p (polyroot),
    weights = p! / (p^2 He_{p-1}(x)^2); weights sum to one (standard normal)."""
    c = hermite_polynomials(p)
    x = np.sort(np.real(np.roots(c[p, ::-1])))
    # polish the roots with Newton steps on He_p (polyroot is accurate to rounding)
    for _ in range(3):
        v = np.polyval(c[p, ::-1], x)
        dv = np.polyval(np.polyder(c[p, ::-1]), x)
        x = x - v / dv
    w = math.factorial(p) / (p * p * np.polyval(c[p - 1, ::-1], x) ** 2)
    return x, w


def gauss_hermite_points_scaled(mean, scale, order=7):
    """gauss_hermite_points_scaled (R/quadrature.R:37-44): n-by-order grid mean + scale*x."""
    x, w = gauss_hermite_points(order)
    mean = np.asarray(mean, dtype=np.float64).ravel()
    scale = np.asarray(scale, dtype=np.float64).ravel()
    return x[None, :] * scale[:, None] + mean[:, None], w


def logsumexp_rows(L, w=None):
    """logsumexp applied per row (R/gp_loo.R:136-144)."""
    c = L.max(axis=1)
    if w is None:
        w = np.ones(L.shape[1])
    with np.errstate(invalid="ignore"):
        return c + np.log((w[None, :] * np.exp(L - c[:, None])).sum(axis=1))


# ----------------------------------------------------------------------------
# Laplace, full method (R/laplace.R:13-39, 274-297)
# ----------------------------------------------------------------------------

def _sub(a, idx):
    return None if a is None else np.asarray(a)[idx]


def _fwd(L, b):
    """forwardsolve(L, b)."""
    return sla.solve_triangular(L, b, lower=True)


def _bwd_t(L, b):
    """backsolve(t(L), b) for a lower L."""
    return sla.solve_triangular(L.T, b, lower=False)


def _bad_site_terms(pred_mean, pred_cov, Vb, zb):
    """The shared algebra of the non-log-concave branches (R/laplace.R:73-98,
    R/ep.R:88-113): the prior of the bad sites given the good ones is
    N(pred_mean, pred_cov); Lk = t(chol(pred_cov)), A = I + Lk^T V^-1 Lk. Returns
    None when chol(A) fails (R returns log_evidence = -Inf there); chol(pred_cov)
    failing is an error, as in R."""
    Lk = sla.cholesky(pred_cov, lower=False).T
    A = np.eye(len(Vb)) + Lk.T @ ((1 / Vb)[:, None] * Lk)
    try:
        A_chol = sla.cholesky(A, lower=False).T
    except np.linalg.LinAlgError:
        return None

    def solve_a(v):  # backsolve(t(A_chol), forwardsolve(A_chol, v))
        return _bwd_t(A_chol, _fwd(A_chol, v))
    alpha2 = _bwd_t(Lk, solve_a(Lk.T @ (zb / Vb)))
    aux = _bwd_t(Lk, _fwd(Lk, pred_mean))
    aux = _bwd_t(Lk, solve_a(Lk.T @ aux))
    f2hat = pred_cov @ (alpha2 + aux)
    return dict(Lk=Lk, A_chol=A_chol, solve_a=solve_a, f2hat=f2hat,
                invC2_V2_logdet=2 * np.log(np.diag(A_chol)).sum())


def laplace_iter_full(lik, K, y, fhat_old, trials=None, offset=None, pobs=None):
    """laplace_iter.method_full (R/laplace.R:13-119): the log-concave branch
    (B factorisation, :21-38) and, when some pseudo-variance is <= 0, the split
    p(y) = p(y_good) p(y_bad | y_good) with an LU of K + diag(V) for the final
    fit (:40-116)."""
    z, V = get_pseudodata_la(lik, fhat_old, y, trials, offset) if pobs is None else pobs
    n = len(z)
    if not np.all(V > 0):
        good = np.nonzero(V > 0)[0]
        bad = np.nonzero(~(V > 0))[0]
        if len(bad) > 500:
            warnings.warn("More than 500 data points with pseudo-variance < 0 (outliers), computation "
                          "getting slow. Check that the model and hyperparameter values are sensible.")
        fit1 = laplace_iter_full(lik, K[np.ix_(good, good)], np.asarray(y)[good], None, _sub(trials, good),
                                 _sub(offset, good), pobs=(z[good], V[good]))
        K21 = K[np.ix_(bad, good)]
        K22 = K[np.ix_(bad, bad)]
        pred_mean = K21 @ fit1["alpha"]
        aux = _fwd(fit1["C_chol"], K21.T)
        pred_cov = K22 - aux.T @ aux
        t = _bad_site_terms(pred_mean, pred_cov, V[bad], z[bad])
        if t is None:
            return dict(fmean=fhat_old, log_evidence=-np.inf)
        df2 = (_fwd(t["Lk"], t["f2hat"] - pred_mean) ** 2).sum()
        log_lik2 = get_loglik(lik, t["f2hat"], np.asarray(y)[bad], _sub(trials, bad), _sub(offset, bad))
        lml2 = log_lik2 - 0.5 * df2 + 0.5 * t["invC2_V2_logdet"]
        C_lu = sla.lu_factor(K + np.diag(V))
        alpha = sla.lu_solve(C_lu, z)
        return dict(fmean=K @ alpha, z=z, V=V, C_lu=C_lu, alpha=alpha,
                    log_evidence=float(fit1["log_evidence"] + lml2))
    sv = np.sqrt(1 / V)
    B = np.eye(n) + sv[:, None] * (K * sv[None, :])
    Lb = sla.cholesky(B, lower=False).T
    C_chol = np.sqrt(V)[:, None] * Lb
    alpha = sla.solve_triangular(C_chol.T, sla.solve_triangular(C_chol, z, lower=True), lower=False)
    fhat_new = K @ alpha
    C_logdet = 2 * np.log(np.diag(C_chol)).sum()
    V_logdet = np.log(V).sum()
    f_invK_f = fhat_new @ alpha
    log_lik = get_loglik(lik, fhat_new, y, trials, offset)
    lml = log_lik - 0.5 * f_invK_f - 0.5 * (C_logdet - V_logdet)
    return dict(fmean=fhat_new, z=z, V=V, C_chol=C_chol, alpha=alpha, log_evidence=float(lml))


def laplace_full(lik, K, y, maxiter=100, tol=1e-4, trials=None, offset=None):
    """laplace.method_full (R/laplace.R:274-297): Newton iteration from f = 0."""
    n = len(y)
    fhat = np.zeros(n)
    if lik.kind == "gaussian":
        maxiter = 1
    it = 0
    for it in range(1, maxiter + 1):
        fit = laplace_iter_full(lik, K, y, fhat, trials, offset)
        diff = np.max(np.abs(fhat - fit["fmean"]))
        fhat = fit["fmean"]
        if diff < tol:
            break
    if maxiter > 1 and it == maxiter:
        warnings.warn("Maximum number of iterations in Laplace reached, max delta f = %g" % diff)
    fit["iters"] = it
    return fit


# ----------------------------------------------------------------------------
# EP, full method (R/lik.R:207-270, R/ep.R:16-49, 286-330)
# ----------------------------------------------------------------------------

def get_tilted_moments(lik, post_mean, post_prec, z_old, P_old, y, quad_order, trials=None, offset=None):
    """get_tilted_moments.lik (R/lik.R:237-270)."""
    cavity_prec = post_prec - P_old
    cavity_mean = 1 / cavity_prec * (post_mean * post_prec - z_old * P_old)
    with np.errstate(invalid="ignore"):
        fgrid, w = gauss_hermite_points_scaled(cavity_mean, np.sqrt(1 / cavity_prec), quad_order)
        loglik = get_loglik(lik, fgrid, y, trials, offset, sum_=False)
        lik_ = np.exp(loglik)
    quad_ok = True
    if np.any(np.isnan(lik_)):
        lik_[np.isnan(lik_)] = 0
        loglik[np.isnan(loglik)] = -np.inf
        quad_ok = False
    log_C = logsumexp_rows(loglik, w)
    C = np.exp(log_C)
    mean_t = (1 / C) * ((fgrid * lik_) @ w)
    s2_t = (1 / C) * (((fgrid - mean_t[:, None]) ** 2 * lik_) @ w)
    return dict(mean_tilted=mean_t, var_tilted=s2_t, log_C=log_C, mean_cavity=cavity_mean,
                var_cavity=1 / cavity_prec, quad_ok=quad_ok)


def get_pseudodata_ep(lik, post_mean, post_prec, z_old, P_old, y, quad_order=11, damping=0.5,
                      trials=None, offset=None):
    """get_pseudodata_ep.lik (R/lik.R:207-232): site update with damping."""
    tm = get_tilted_moments(lik, post_mean, post_prec, z_old, P_old, y, quad_order, trials, offset)
    with np.errstate(divide="ignore", invalid="ignore"):
        P_new = 1 / tm["var_tilted"] - 1 / tm["var_cavity"]
        nu_new = tm["mean_tilted"] / tm["var_tilted"] - tm["mean_cavity"] / tm["var_cavity"]
        nu_old = z_old * P_old
        nu_new = damping * nu_new + (1 - damping) * nu_old
        P_new = damping * P_new + (1 - damping) * P_old
        return dict(z=(1 / P_new) * nu_new, var=1 / P_new, log_C=tm["log_C"],
                    mean_cavity=tm["mean_cavity"], var_cavity=tm["var_cavity"], quad_ok=tm["quad_ok"])


def ep_iter_full(lik, K, y, fmean_old, fvar_old, z_old, P_old, quad_order, damping,
                 trials=None, offset=None, po=None):
    """ep_iter.method_full (R/ep.R:16-145): the log-concave branch (:33-49) and, when
    some site variance is <= 0, the split p(y_good) p(y_bad | y_good) with an LU of
    K + diag(V) for the final fit (:50-138)."""
    if po is None:
        po = get_pseudodata_ep(lik, fmean_old, 1 / fvar_old, z_old, P_old, y, quad_order, damping,
                               trials, offset)
    z, V = po["z"], po["var"]
    if np.any(np.isnan(V) | np.isnan(z)):
        return dict(fmean=fmean_old, log_evidence=-np.inf, nan=True)
    if not np.all(V > 0):
        good = np.nonzero(V > 0)[0]
        bad = np.nonzero(~(V > 0))[0]
        if len(bad) > 500:
            warnings.warn("More than 500 data points with pseudo-variance < 0 (outliers), computation "
                          "getting slow. Check that the model and hyperparameter values are sensible.")
        po1 = dict(z=z[good], var=V[good], log_C=po["log_C"][good], mean_cavity=po["mean_cavity"][good],
                   var_cavity=po["var_cavity"][good], quad_ok=po["quad_ok"])
        fit1 = ep_iter_full(lik, K[np.ix_(good, good)], np.asarray(y)[good], None, None, None, None,
                            quad_order, damping, _sub(trials, good), _sub(offset, good), po=po1)
        K21 = K[np.ix_(bad, good)]
        K22 = K[np.ix_(bad, bad)]
        pred_mean = K21 @ fit1["alpha"]
        aux = _fwd(fit1["C_chol"], K21.T)
        pred_cov = K22 - aux.T @ aux
        Vb, zb = V[bad], z[bad]
        t = _bad_site_terms(pred_mean, pred_cov, Vb, zb)
        if t is None:
            return dict(fmean=np.inf, log_evidence=-np.inf)
        d = pred_mean - zb
        df2 = d @ _bwd_t(t["Lk"], t["solve_a"](t["Lk"].T @ (d / Vb)))
        vc, mc = po["var_cavity"], po["mean_cavity"]
        lml2 = (-0.5 * df2 + 0.5 * t["invC2_V2_logdet"] + po["log_C"][bad].sum()
                + 0.5 * np.log((vc[bad] + Vb) / Vb).sum() + 0.5 * ((mc[bad] - zb) ** 2 / (vc[bad] + Vb)).sum())
        C_lu = sla.lu_factor(K + np.diag(V))
        alpha = sla.lu_solve(C_lu, z)
        fvar = V * np.diag(sla.lu_solve(C_lu, K))
        return dict(fmean=K @ alpha, fvar=fvar, cavity_mean=mc, cavity_var=vc, z=z, P=1 / V, V=V,
                    C_lu=C_lu, alpha=alpha, log_evidence=float(fit1["log_evidence"] + lml2),
                    quad_ok=po["quad_ok"])
    n = len(z)
    sv = np.sqrt(1 / V)
    B = np.eye(n) + sv[:, None] * (K * sv[None, :])
    C_chol = np.sqrt(V)[:, None] * sla.cholesky(B, lower=False).T
    alpha = sla.solve_triangular(C_chol.T, sla.solve_triangular(C_chol, z, lower=True), lower=False)
    fmean_new = K @ alpha
    CinvK = sla.solve_triangular(C_chol.T, sla.solve_triangular(C_chol, K, lower=True), lower=False)
    fvar_new = V * np.diag(CinvK)
    C_logdet = 2 * np.log(np.diag(C_chol)).sum()
    z_invC_z = z @ alpha
    vc, mc = po["var_cavity"], po["mean_cavity"]
    lml = (-0.5 * C_logdet - 0.5 * z_invC_z + po["log_C"].sum()
           + 0.5 * np.log(vc + V).sum() + 0.5 * ((mc - z) ** 2 / (vc + V)).sum())
    return dict(fmean=fmean_new, fvar=fvar_new, cavity_mean=mc, cavity_var=vc, z=z, P=1 / V,
                V=V, C_chol=C_chol, alpha=alpha, log_evidence=float(lml), quad_ok=po["quad_ok"])


def ep_full(lik, K, y, maxiter=300, tol=1e-4, damping=0.9, damping_min=0.1, quad_order=11,
            trials=None, offset=None):
    """ep.method_full (R/ep.R:286-330): parallel EP with adaptive damping."""
    n = len(y)
    P_old = np.zeros(n)
    z_old = np.zeros(n)
    fmean_old = np.zeros(n)
    fvar_old = np.diag(K).copy()
    diff_old = np.inf
    damp = damping
    it = 0
    diff_new = np.inf
    fit = None
    for it in range(1, maxiter + 1):
        fit = ep_iter_full(lik, K, y, fmean_old, fvar_old, z_old, P_old, quad_order, damp, trials, offset)
        if fit.get("nan"):
            return fit
        diff_new = np.max(np.abs(fmean_old - fit["fmean"]))
        if diff_new > diff_old:
            damp = damp * damping
            continue
        damp = max(damp, damping_min)
        if "fvar" not in fit:  # R goes on with fvar_old = NULL and errors in the next sweep
            raise ValueError("EP: the first sweep has an improper posterior for the bad sites")
        fmean_old, fvar_old, z_old, P_old = fit["fmean"], fit["fvar"], fit["z"], fit["P"]
        diff_old = diff_new
        if diff_new < tol:
            break
    if maxiter > 1 and it == maxiter:
        fit["log_evidence"] = -np.inf
        warnings.warn("Maximum number of iterations in EP reached, max delta f = %g" % diff_new)
    if fit.get("quad_ok") is False:
        fit["log_evidence"] = -np.inf
    fit["iters"] = it
    return fit


# ----------------------------------------------------------------------------
# inversion lemma (R/linear_algebra.R:3-143) and FITC (R/gp_fit.R:101-123,163-188,
# R/laplace.R:122-152,299-325, R/ep.R:148-185,333-374)
# ----------------------------------------------------------------------------

def inv_lemma_get(K, U, D, logdet=True):
    """inv_lemma_get (R/linear_algebra.R:3-43) with V = t(U)."""
    D = np.asarray(D, dtype=np.float64).ravel()
    inv_D_U = U / D[:, None]
    VDU = U.T @ inv_D_U
    VDU = 0.5 * (VDU + VDU.T)
    L = sla.cholesky(K + VDU, lower=False).T
    ld = None
    if logdet:
        ld = np.log(D).sum() - 2 * np.log(np.diag(sla.cholesky(K, lower=False))).sum() \
            + 2 * np.log(np.diag(L)).sum()
    return dict(chol=L, D=D, inv_D_U=inv_D_U, logdet=ld)


def _chol_solve_lower(L, b):
    return sla.solve_triangular(L.T, sla.solve_triangular(L, b, lower=True), lower=False)


def inv_lemma_solve(obj, rhs, lhs=None, rhs_diag=False, lhs_diag=False, diag_only=False):
    """inv_lemma_solve (R/linear_algebra.R:45-126), the cases the hot path uses."""
    D, iDU, L = obj["D"], obj["inv_D_U"], obj["chol"]
    if lhs is None:
        if rhs_diag:
            aux_right = iDU.T * rhs[None, :]
            return np.diag(rhs / D) - iDU @ _chol_solve_lower(L, aux_right)
        aux_right = iDU.T @ rhs
        aux_left = rhs / D if rhs.ndim == 1 else rhs / D[:, None]
        return aux_left - iDU @ _chol_solve_lower(L, aux_right)
    if rhs_diag:
        aux_right = iDU.T * rhs[None, :]
        if lhs_diag:
            if diag_only:
                return lhs / D * rhs - ((lhs[:, None] * iDU).T * _chol_solve_lower(L, aux_right)).sum(0)
            return np.diag(lhs / D * rhs) - (lhs[:, None] * iDU) @ _chol_solve_lower(L, aux_right)
        return lhs * (rhs / D)[None, :] - (lhs @ iDU) @ _chol_solve_lower(L, aux_right)
    aux_right = iDU.T @ rhs
    if lhs_diag:
        return (lhs / D)[:, None] * rhs - (lhs[:, None] * iDU) @ _chol_solve_lower(L, aux_right)
    return lhs @ (rhs / D[:, None]) - (lhs @ iDU) @ _chol_solve_lower(L, aux_right)


def fitc_prepare(cfs, x, z, jitter):
    """The FITC set-up of fit_laplace.method_fitc / fit_ep.method_fitc (R/gp_fit.R:101-111,
    163-173)."""
    M = z.shape[0]
    Kz = eval_cf(cfs, z, z) + jitter * np.eye(M)
    Kxz = eval_cf(cfs, x, z)
    Kz_chol = sla.cholesky(Kz, lower=False).T
    K_diag = eval_cf(cfs, x, x, diag_only=True) + jitter
    D = K_diag - (sla.solve_triangular(Kz_chol, Kxz.T, lower=True) ** 2).sum(0)
    return Kz, Kxz, Kz_chol, K_diag, D


def _fitc_bad_prior(Kz_chol, Kxz, D, good, bad, fit1):
    """Prior of the bad sites given the good ones under FITC (R/laplace.R:179-186,
    R/ep.R:219-226): K21 through the inducing inputs, the bad sites' own FITC prior
    covariance, and the lemma solve with the good fit's C_inv."""
    Lb = _fwd(Kz_chol, Kxz[bad].T)
    K21 = Lb.T @ _fwd(Kz_chol, Kxz[good].T)
    prior_cov = Lb.T @ Lb + np.diag(D[bad])
    pred_mean = K21 @ fit1["alpha"]
    pred_cov = prior_cov - K21 @ inv_lemma_solve(fit1["C_inv"], K21.T)
    return pred_mean, pred_cov


def laplace_iter_fitc(lik, Kz, Kz_chol, Kxz, D, y, fhat_old, trials=None, offset=None, pobs=None):
    """laplace_iter.method_fitc (R/laplace.R:122-238): the log-concave branch
    (:136-150) and, when some pseudo-variance is <= 0, the good / bad split with the
    lemma of the whole data (S = D + V, no log-determinant) for the final fit (:151-231)."""
    z, V = get_pseudodata_la(lik, fhat_old, y, trials, offset) if pobs is None else pobs
    if not np.all(V > 0):
        good = np.nonzero(V > 0)[0]
        bad = np.nonzero(~(V > 0))[0]
        if len(bad) > 500:
            warnings.warn("More than 500 data points with pseudo-variance < 0 (outliers), computation "
                          "getting slow. Check that the model and hyperparameter values are sensible.")
        fit1 = laplace_iter_fitc(lik, Kz, Kz_chol, Kxz[good], D[good], np.asarray(y)[good], None,
                                 _sub(trials, good), _sub(offset, good), pobs=(z[good], V[good]))
        pred_mean, pred_cov = _fitc_bad_prior(Kz_chol, Kxz, D, good, bad, fit1)
        t = _bad_site_terms(pred_mean, pred_cov, V[bad], z[bad])
        if t is None:
            return dict(fmean=fhat_old, log_evidence=-np.inf)
        df2 = (_fwd(t["Lk"], t["f2hat"] - pred_mean) ** 2).sum()
        log_lik2 = get_loglik(lik, t["f2hat"], np.asarray(y)[bad], _sub(trials, bad), _sub(offset, bad))
        lpu2 = float(log_lik2 - 0.5 * df2)
        lml2 = log_lik2 - 0.5 * df2 + 0.5 * t["invC2_V2_logdet"]
        Ci = inv_lemma_get(Kz, Kxz, D + V, logdet=False)
        alpha = inv_lemma_solve(Ci, z)
        fhat = Kxz @ _chol_solve_lower(Kz_chol, Kxz.T @ alpha) + D * alpha
        return dict(fmean=fhat, z=z, V=V, Kz=Kz, Kxz=Kxz, Kz_chol=Kz_chol, C_inv=Ci, diag=D, alpha=alpha,
                    log_evidence=float(fit1["log_evidence"] + lml2),
                    log_post_unnorm=float(fit1["log_post_unnorm"] + lpu2))
    S = D + V
    Ci = inv_lemma_get(Kz, Kxz, S)
    alpha = inv_lemma_solve(Ci, z)
    fhat = Kxz @ _chol_solve_lower(Kz_chol, Kxz.T @ alpha) + D * alpha
    invC_V_logdet = np.log(V).sum() - Ci["logdet"]
    f_invK_f = fhat @ alpha
    log_lik = get_loglik(lik, fhat, y, trials, offset)
    lml = log_lik - 0.5 * f_invK_f + 0.5 * invC_V_logdet
    return dict(fmean=fhat, z=z, V=V, Kz=Kz, Kxz=Kxz, Kz_chol=Kz_chol, C_inv=Ci, diag=D, alpha=alpha,
                log_evidence=float(lml), log_post_unnorm=float(log_lik - 0.5 * f_invK_f))


def laplace_fitc(lik, Kz, Kz_chol, Kxz, D, y, maxiter=100, tol=1e-4, trials=None, offset=None):
    """laplace.method_fitc (R/laplace.R:299-325): stops on |delta log_post_unnorm| < tol."""
    n = len(y)
    fhat = np.zeros(n)
    if lik.kind == "gaussian":
        maxiter = 1
    old = -np.inf
    it = 0
    for it in range(1, maxiter + 1):
        fit = laplace_iter_fitc(lik, Kz, Kz_chol, Kxz, D, y, fhat, trials, offset)
        fhat = fit["fmean"]
        d = fit["log_post_unnorm"] - old
        old = fit["log_post_unnorm"]
        if abs(d) < tol:
            break
    if maxiter > 1 and it == maxiter:
        warnings.warn("Maximum number of iterations in Laplace reached")
    fit["iters"] = it
    return fit


def ep_iter_fitc(lik, Kz, Kz_chol, Kxz, D, y, fmean_old, fvar_old, z_old, P_old, quad_order, damping,
                 trials=None, offset=None, po=None):
    """ep_iter.method_fitc (R/ep.R:148-279): the log-concave branch (:167-185) and,
    when some site variance is <= 0, the good / bad split with the lemma of the whole
    data for the final fit (:186-272)."""
    if po is None:
        po = get_pseudodata_ep(lik, fmean_old, 1 / fvar_old, z_old, P_old, y, quad_order, damping,
                               trials, offset)
    z, V = po["z"], po["var"]
    if np.any(np.isnan(V) | np.isnan(z)):
        return dict(fmean=fmean_old, log_evidence=-np.inf, nan=True)
    if not np.all(V > 0):
        good = np.nonzero(V > 0)[0]
        bad = np.nonzero(~(V > 0))[0]
        if len(bad) > 500:
            warnings.warn("More than 500 data points with pseudo-variance < 0 (outliers), computation "
                          "getting slow. Check that the model and hyperparameter values are sensible.")
        po1 = dict(z=z[good], var=V[good], log_C=po["log_C"][good], mean_cavity=po["mean_cavity"][good],
                   var_cavity=po["var_cavity"][good], quad_ok=po["quad_ok"])
        fit1 = ep_iter_fitc(lik, Kz, Kz_chol, Kxz[good], D[good], np.asarray(y)[good], None, None, None, None,
                            quad_order, damping, _sub(trials, good), _sub(offset, good), po=po1)
        pred_mean, pred_cov = _fitc_bad_prior(Kz_chol, Kxz, D, good, bad, fit1)
        Vb, zb = V[bad], z[bad]
        t = _bad_site_terms(pred_mean, pred_cov, Vb, zb)
        if t is None:
            return dict(fmean=np.inf, log_evidence=-np.inf)
        d = pred_mean - zb
        df2 = d @ _bwd_t(t["Lk"], t["solve_a"](t["Lk"].T @ (d / Vb)))
        vc, mc = po["var_cavity"], po["mean_cavity"]
        lml2 = (-0.5 * df2 + 0.5 * t["invC2_V2_logdet"] + po["log_C"][bad].sum()
                + 0.5 * np.log((vc[bad] + Vb) / Vb).sum() + 0.5 * ((mc[bad] - zb) ** 2 / (vc[bad] + Vb)).sum())
        Ci = inv_lemma_get(Kz, Kxz, D + V, logdet=False)
        alpha = inv_lemma_solve(Ci, z)
        inv_Kz_Kzx = _chol_solve_lower(Kz_chol, Kxz.T)
        aux = inv_lemma_solve(Ci, V, inv_Kz_Kzx, rhs_diag=True)
        fvar = (Kxz.T * aux).sum(0) + inv_lemma_solve(Ci, V, D, rhs_diag=True, lhs_diag=True, diag_only=True)
        fmean = Kxz @ _chol_solve_lower(Kz_chol, Kxz.T @ alpha) + D * alpha
        return dict(fmean=fmean, fvar=fvar, cavity_mean=mc, cavity_var=vc, z=z, P=1 / V, V=V, Kz=Kz,
                    Kxz=Kxz, Kz_chol=Kz_chol, C_inv=Ci, diag=D, alpha=alpha,
                    log_evidence=float(fit1["log_evidence"] + lml2), quad_ok=po["quad_ok"])
    S = D + V
    Ci = inv_lemma_get(Kz, Kxz, S)
    alpha = inv_lemma_solve(Ci, z)
    inv_Kz_Kzx = _chol_solve_lower(Kz_chol, Kxz.T)
    aux = inv_lemma_solve(Ci, V, inv_Kz_Kzx, rhs_diag=True)
    diag1 = (Kxz.T * aux).sum(0)
    diag2 = inv_lemma_solve(Ci, V, D, rhs_diag=True, lhs_diag=True, diag_only=True)
    fvar = diag1 + diag2
    fmean = Kxz @ _chol_solve_lower(Kz_chol, Kxz.T @ alpha) + D * alpha
    vc, mc = po["var_cavity"], po["mean_cavity"]
    lml = (-0.5 * Ci["logdet"] - 0.5 * z @ alpha + po["log_C"].sum()
           + 0.5 * np.log(vc + V).sum() + 0.5 * ((mc - z) ** 2 / (vc + V)).sum())
    return dict(fmean=fmean, fvar=fvar, cavity_mean=mc, cavity_var=vc, z=z, P=1 / V, V=V, Kz=Kz,
                Kxz=Kxz, Kz_chol=Kz_chol, C_inv=Ci, diag=D, alpha=alpha, log_evidence=float(lml),
                quad_ok=po["quad_ok"])


def ep_fitc(lik, Kz, Kz_chol, Kxz, K_diag, D, y, damping=0.9, damping_min=0.1, maxiter=100, tol=1e-3,
            quad_order=11, trials=None, offset=None):
    """ep.method_fitc (R/ep.R:333-374)."""
    n = len(y)
    P_old = np.zeros(n)
    z_old = np.zeros(n)
    fmean_old = np.zeros(n)
    fvar_old = K_diag.copy()
    diff_old = np.inf
    damp = damping
    it = 0
    diff_new = np.inf
    fit = None
    for it in range(1, maxiter + 1):
        fit = ep_iter_fitc(lik, Kz, Kz_chol, Kxz, D, y, fmean_old, fvar_old, z_old, P_old, quad_order,
                           damp, trials, offset)
        if fit.get("nan"):
            return fit
        diff_new = np.max(np.abs(fmean_old - fit["fmean"]))
        if diff_new > diff_old:
            damp = damp * damping
            continue
        damp = max(damp, damping_min)
        if "fvar" not in fit:  # R goes on with fvar_old = NULL and errors in the next sweep
            raise np.linalg.LinAlgError("EP: the first sweep has an improper posterior for the bad sites")
        fmean_old, fvar_old, z_old, P_old = fit["fmean"], fit["fvar"], fit["z"], fit["P"]
        diff_old = diff_new
        if diff_new < tol:
            break
    if maxiter > 1 and it == maxiter:
        fit["log_evidence"] = -np.inf
    if fit.get("quad_ok") is False:
        fit["log_evidence"] = -np.inf
    fit["iters"] = it
    return fit


# ----------------------------------------------------------------------------
# random features: method_rf / method_rbf (R/method.R:129-139, R/cf.R:532-817,
# R/laplace.R:241-266, 327-355, R/gp_pred.R:186-200, 298-318, R/gp_draw.R:87-169).
# R draws the frequencies / centres after set.seed(seed) in every feature-map
# constructor; numpy's default_rng(seed), restarted for every covariance function
# (and every factor of a product), stands in for that stream here: the same
# shapes, order and distributions, other numbers.
# ----------------------------------------------------------------------------

def check_num_basis(cfs, num_basis, num_inputs=None):
    """check_num_basis (R/gp.R:211-233)."""
    if num_basis is None:
        return None
    nb = list(np.atleast_1d(np.asarray(num_basis, dtype=object)))
    if len(nb) == 1:
        nb = nb * len(cfs)
    if len(nb) != len(cfs):
        raise ValueError("The length of num_basis must match to the number of covariance functions.")
    for k, c in enumerate(cfs):
        if c.kind == "const":
            nb[k] = 1
        elif c.kind == "lin":
            nb[k] = len(c.vars) if c.vars is not None else num_inputs
    return nb


def _n_inputs(cf, num_inputs):
    return len(cf.vars) if cf.vars is not None else num_inputs


def rf_featmap(cf, num_feat, num_inputs, seed):
    """rf_featmap.cf_* (R/cf.R:553-695)."""
    if cf.kind == "const":
        return lambda x: cf.magn * np.ones((as_matrix(x).shape[0], 1))
    if cf.kind == "lin":
        return lambda x: cf.magn * prepare_inputmat(cf, x)
    if cf.kind in ("matern32", "matern52"):
        raise ValueError("Random Fourier features for Matern kernels not implemented yet.")
    if cf.kind == "sexp":
        q = _n_inputs(cf, num_inputs)
        if num_feat % 2 == 1:
            raise ValueError("number of features must be an even number.")
        m = num_feat // 2
        scale = 1 / cf.lscale
        w = np.random.default_rng(seed).standard_normal(m * q).reshape(m, q).T * scale

        def fm(x):
            h = prepare_inputmat(cf, x) @ w
            return cf.magn * math.sqrt(1 / m) * np.hstack([np.cos(h), np.sin(h)])
        return fm
    if cf.kind == "nn":
        q = _n_inputs(cf, num_inputs)
        m = num_feat
        rng = np.random.default_rng(seed)
        w = rng.standard_normal(m * q).reshape(m, q).T * cf.sigma
        w0 = rng.standard_normal(m).reshape(1, m) * cf.sigma0 * cf.sigma
        w_aug = np.vstack([w0, w])

        def fm(x):
            x = prepare_inputmat(cf, x)
            x_aug = np.hstack([np.ones((x.shape[0], 1)), x])
            return cf.magn / math.sqrt(m) * sps.erf(x_aug @ w_aug)
        return fm
    if cf.kind == "periodic":
        q = _n_inputs(cf, num_inputs)
        base = rf_featmap(cf.base, num_feat, 2 * q, seed)

        def fm(x):
            x = prepare_inputmat(cf, x)
            w = 2 * math.pi / cf.period
            return base(np.hstack([np.sin(w * x), np.cos(w * x)]))
        return fm
    if cf.kind == "prod":
        if any(c.kind in ("const", "lin") for c in cf.cfs):
            raise ValueError("Random features for product kernel containing constant or linear kernel "
                             "not implemented yet.")
        maps = [rf_featmap(c, num_feat, num_inputs, seed) for c in cf.cfs]

        def fm(x):
            z = 1
            for mp in maps:
                z = z * mp(x)
            return z
        return fm
    raise ValueError(cf.kind)


def rbf_featmap(cf, num_feat, num_inputs, x, seed):
    """rbf_featmap.cf_* (R/cf.R:722-817). Centres are training inputs sampled without
    replacement (R's sample(n, num_feat)) from the columns the term uses."""
    if cf.kind in ("const", "lin"):
        return rf_featmap(cf, num_feat, num_inputs, seed)
    if cf.kind == "sexp":
        if x is None:
            raise ValueError("Cannot get RBF featuremap if inputs are not given.")
        xs = as_matrix(x)
        if cf.vars is not None:
            xs = xs[:, list(cf.vars)]
        ind = np.random.default_rng(seed).choice(xs.shape[0], num_feat, replace=False)
        centers = xs[ind]

        def fm(xx):
            xx = prepare_inputmat(cf, xx)
            z = np.empty((xx.shape[0], num_feat))
            for j in range(num_feat):
                z[:, j] = np.exp(-((xx - centers[j]) ** 2).sum(1) / cf.lscale ** 2)
            return cf.magn * math.sqrt(1 / num_feat) * z
        return fm
    if cf.kind == "periodic":
        q = _n_inputs(cf, num_inputs)
        xs = as_matrix(x)
        if cf.vars is not None:
            xs = xs[:, list(cf.vars)]
        w = 2 * math.pi / cf.period
        base = rbf_featmap(cf.base, num_feat, 2 * q, np.hstack([np.sin(w * xs), np.cos(w * xs)]), seed)

        def fm(xx):
            xx = prepare_inputmat(cf, xx)
            return base(np.hstack([np.sin(w * xx), np.cos(w * xx)]))
        return fm
    if cf.kind == "prod":
        if any(c.kind in ("const", "lin") for c in cf.cfs):
            raise ValueError("RBF features for product kernel containing constant or linear kernel "
                             "not implemented yet.")
        maps = [rbf_featmap(c, num_feat, num_inputs, x, seed) for c in cf.cfs]

        def fm(xx):
            z = 1
            for mp in maps:
                z = z * mp(xx)
            return z
        return fm
    raise ValueError("no RBF feature map for cf_%s" % cf.kind)


def get_featuremap(gp, num_inputs):
    """get_featuremap.gp + rf_featmap.list / rbf_featmap.list (R/gp.R:171-189,
    R/cf.R:534-551, 703-720): the features of the selected cfs, side by side."""
    me = gp.method
    nb = check_num_basis(gp.cfs, me.num_basis, num_inputs)
    if me.kind == "rf":
        maps = [rf_featmap(c, nb[k], num_inputs, me.seed) for k, c in enumerate(gp.cfs)]
    else:
        if getattr(gp, "x", None) is None:
            raise ValueError("Cannot compute RBF feature map when the x matrix is not known.")
        maps = [rbf_featmap(c, nb[k], num_inputs, gp.x, me.seed) for k, c in enumerate(gp.cfs)]

    def featuremap(x, cfind=None):
        idx = range(len(maps)) if cfind is None else cfind
        return np.hstack([maps[k](x) for k in idx])
    return featuremap


def get_weight_inds(gp, cfind=None):
    """get_weight_inds (R/gp.R:235-245), 0-based."""
    ends = np.concatenate([[0], np.cumsum(gp.method.num_basis)]).astype(int)
    idx = range(len(gp.cfs)) if cfind is None else cfind
    return np.concatenate([np.arange(ends[k], ends[k + 1]) for k in idx])


def laplace_iter_rf(lik, Z, y, fhat_old, trials=None, offset=None):
    """laplace_iter.method_rf (R/laplace.R:241-262)."""
    z, V = get_pseudodata_la(lik, fhat_old, y, trials, offset)
    n = len(z)
    d = Z.shape[1]
    H = Z.T @ (Z / V[:, None])
    L = np.linalg.cholesky(H + np.eye(d))
    what = _bwd_t(L, _fwd(L, Z.T @ (z / V)))
    wcov = sla.solve_triangular(L, sla.solve_triangular(L, np.eye(d), lower=True), lower=True, trans="T")
    wcov_logdet = -2 * np.sum(np.log(np.diag(L)))
    fhat_new = Z @ what
    log_prior = -0.5 * d * math.log(2 * math.pi) - 0.5 * np.sum(what ** 2)
    log_lik = get_loglik(lik, fhat_new, y, trials, offset)
    log_evidence = 0.5 * n * math.log(2 * math.pi) + 0.5 * wcov_logdet + log_prior + log_lik
    return dict(fmean=fhat_new, wmean=what, wcov=wcov, z=z, V=V, log_evidence=log_evidence)


def laplace_rf(lik, Z, y, maxiter=100, tol=1e-4, trials=None, offset=None):
    """laplace.method_rf (R/laplace.R:327-351)."""
    n = len(y)
    fhat = np.zeros(n)
    if lik.kind == "gaussian":
        maxiter = 1
    for it in range(1, maxiter + 1):
        fit = laplace_iter_rf(lik, Z, y, fhat, trials, offset)
        fhat_new = Z @ fit["wmean"]
        diff = np.max(np.abs(fhat - fhat_new))
        fhat = fhat_new
        if diff < tol:
            break
    if maxiter > 1 and it == maxiter:
        warnings.warn("Maximum number of iterations in Laplace reached, max delta f = %g" % diff)
    fit["iters"] = it
    return fit


def gp_pred_post_rf(gp, xt, var=False, cfind=None):
    """gp_pred_post.method_rf (R/gp_pred.R:298-314)."""
    zt = get_featuremap(gp, xt.shape[1])(xt, cfind)
    inds = get_weight_inds(gp, cfind)
    pred = dict(mean=zt @ gp.fit["wmean"][inds])
    if var:
        wcov = gp.fit["wcov"][np.ix_(inds, inds)]
        pred["var"] = np.einsum("ij,jk,ik->i", zt, wcov, zt)
    return pred


def gp_draw_rf(gp, xt, z, cfind=None):
    """gp_draw_prior / gp_draw_analytic.method_rf (R/gp_draw.R:87-103, 145-163) with the
    standard normals z (features x draws) given: zt w, w = z (prior) or
    wmean + t(chol(wcov)) z (posterior, mvnrnd R/gp_draw.R:182-188)."""
    xt = as_matrix(xt)
    zt = get_featuremap(gp, xt.shape[1])(xt, cfind)
    if getattr(gp, "fit", None) is None:
        return zt @ z
    inds = get_weight_inds(gp, cfind)
    wmean = gp.fit["wmean"][inds]
    wcov = gp.fit["wcov"][np.ix_(inds, inds)]
    return zt @ (wmean[:, None] + np.linalg.cholesky(wcov) @ z)


def method_rf(num_basis=400, seed=12345):
    return SimpleNamespace(kind="rf", num_basis=num_basis, seed=seed)


def method_rbf(num_basis=400, seed=12345):
    return SimpleNamespace(kind="rbf", num_basis=num_basis, seed=seed)


# ----------------------------------------------------------------------------
# gp_fit / gp_energy / gp_pred / gp_loo (R/gp_fit.R:54-188, R/gp.R:138-147,
# R/gp_pred.R:88-296, R/gp_loo.R:73-133)
# ----------------------------------------------------------------------------

def gp_fit(gp, x, y, trials=None, offset=None, jitter=None, threads=1):
    """gp_fit (R/gp_fit.R:54-60) -> fit_laplace/fit_ep.method_full/fitc. threads > 1
    evaluates the covariance matrix in parallel row blocks (same values)."""
    x = as_matrix(x)
    y = np.asarray(y, dtype=np.float64)
    jitter = 1e-6 if jitter is None else jitter
    learn_scales(gp.cfs, x)
    n = len(y)
    ap, me = gp.approx, gp.method
    if ap.kind == "ep" and gp.lik.kind == "gaussian":
        raise ValueError("approx_ep disabled for lik_gaussian")
    if me.kind == "full":
        K = eval_cf(gp.cfs, x, x, threads=threads)
        K[np.diag_indices(n)] += jitter  # + jitter * diag(n) (R/gp_fit.R:95)
        if ap.kind == "laplace":
            fit = laplace_full(gp.lik, K, y, ap.maxiter, ap.tol, trials, offset)
        else:
            fit = ep_full(gp.lik, K, y, maxiter=ap.maxiter, tol=1e-4, damping=ap.damping,
                          damping_min=0.1, quad_order=ap.quad_order, trials=trials, offset=offset)
    elif me.kind == "fitc":
        z = as_matrix(me.inducing)
        try:
            Kz, Kxz, Kz_chol, K_diag, D = fitc_prepare(gp.cfs, x, z, jitter)
            if ap.kind == "laplace":
                fit = laplace_fitc(gp.lik, Kz, Kz_chol, Kxz, D, y, ap.maxiter, ap.tol, trials, offset)
            else:
                fit = ep_fitc(gp.lik, Kz, Kz_chol, Kxz, K_diag, D, y, damping=ap.damping, damping_min=0.1,
                              maxiter=ap.maxiter, quad_order=ap.quad_order, trials=trials, offset=offset)
        except np.linalg.LinAlgError:
            fit = dict(log_evidence=-np.inf)
    elif me.kind in ("rf", "rbf"):
        # fit_laplace.method_rf / method_rbf (R/gp_fit.R:125-141)
        if ap.kind != "laplace":
            raise ValueError("approx_ep is not available for method_%s" % me.kind)
        gp.x = x
        featuremap = get_featuremap(gp, x.shape[1])
        me.num_basis = check_num_basis(gp.cfs, me.num_basis, x.shape[1])
        fit = laplace_rf(gp.lik, featuremap(x), y, ap.maxiter, ap.tol, trials, offset)
    else:
        raise ValueError(me.kind)
    gp.x = x
    gp.fit = fit
    gp.fit_jitter = jitter
    gp.fitted = True
    return gp


def gp_energy(gp, include_prior=True):
    """gp_energy (R/gp.R:138-147)."""
    if getattr(gp, "fit", None) is None:
        raise RuntimeError("The GP must be fitted. Call gp_fit first.")
    if not gp.fitted:
        raise RuntimeError("The GP object seems to contain a posterior fit, but is not refitted")
    e = -gp.fit["log_evidence"]
    if include_prior:
        e = e - lpdf_prior(gp)
    return e


# ----------------------------------------------------------------------------
# energy gradient. The reference has none: gp_optim minimises gp_energy with
# Nelder-Mead (R/gp_optim.R:76-94). This is restated from the mathematics to
# check the device gradient: d log_evidence / d log(theta) of a Gaussian
# full-method fit is (1/2) tr((alpha alpha^T - C^-1) dC/dlog(theta)) with
# C = K + jitter I + sigma^2 I. The analytic derivatives of each covariance
# function are pinned by complex-step differentiation of eval_cf itself
# (Squire & Trapp 1998: df/dt = Im f(t + ih) / h, exact to rounding).
# ----------------------------------------------------------------------------

_STATIONARY = ("sexp", "matern32", "matern52")


def _nn_parts(cf, x1, x2):
    """cf_nn_c's intermediate quantities (src/cf.cpp:148-160): A, B, C, q, u, K."""
    s0 = cf.sigma0 * cf.sigma0 * cf.sigma * cf.sigma
    a1, a2 = x1 * cf.sigma, x2 * cf.sigma
    A = s0 + a1 @ a2.T
    B = (s0 + (a1 * a1).sum(1))[:, None]
    Cc = (s0 + (a2 * a2).sum(1))[None, :]
    q = np.sqrt((1 + 2 * B) * (1 + 2 * Cc))
    u = 2 * A / q
    K = cf.magn ** 2 * (2.0 / math.pi) * np.arcsin(u)
    return A, B, Cc, q, u, K


def _stationary_parts(cf, x1, x2):
    """K, dK/dlog(lscale) and dK/d(r^2) of sexp / matern32 / matern52 (src/cf.cpp:35-117)."""
    r2 = _sqdist(x1, x2)
    m2, ls = cf.magn ** 2, cf.lscale
    if cf.kind == "sexp":
        K = m2 * np.exp(-0.5 * r2 / (ls * ls))
        return K, K * r2 / (ls * ls), -0.5 * K / (ls * ls)
    c = math.sqrt(3.0 if cf.kind == "matern32" else 5.0) / ls
    a = c * np.sqrt(r2)
    e = np.exp(-a)
    if cf.kind == "matern32":
        return m2 * (1 + a) * e, m2 * a * a * e, -0.5 * m2 * c * c * e
    return (m2 * (1 + a + a * a / 3) * e, m2 * a * a * (1 + a) / 3 * e,
            -m2 * c * c * (1 + a) * e / 6)


def kernel_and_grads(cf, x1, x2):
    """K(x1, x2) of one covariance function and dK/dlog(theta) for each of its free
    parameters, in get_param order (R/cf.R:313-344)."""
    if cf.kind == "prod":
        parts = [kernel_and_grads(c, x1, x2) for c in cf.cfs]
        K = 1.0
        for Kc, _ in parts:
            K = K * Kc
        grads = []
        for i, (_, gc) in enumerate(parts):
            others = 1.0
            for j, (Ko, _) in enumerate(parts):
                if j != i:
                    others = others * Ko
            grads += [g * others for g in gc]
        return K, grads
    x1 = prepare_inputmat(cf, x1)
    x2 = prepare_inputmat(cf, x2)
    n1, n2 = x1.shape[0], x2.shape[0]
    if cf.kind == "periodic":
        w = 2 * math.pi / cf.period
        t1 = np.hstack([np.sin(w * x1), np.cos(w * x1)])
        t2 = np.hstack([np.sin(w * x2), np.cos(w * x2)])
        K, gb = kernel_and_grads(cf.base, t1, t2)
        if _is_fixed(cf, "period"):
            return K, gb
        # S = sum_k d_k sin(w d_k), d = x1_k - x2_k; dw/dlog(period) = -w
        S = np.zeros((n1, n2))
        for k in range(x1.shape[1]):
            d = x1[:, k][:, None] - x2[:, k][None, :]
            S += d * np.sin(w * d)
        b = cf.base
        if b.kind == "const":
            dp = np.zeros((n1, n2))
        elif b.kind == "lin":  # K = m^2 sum_k cos(w d_k)
            dp = b.magn ** 2 * w * S
        elif b.kind in _STATIONARY:  # r^2 = sum_k 2 - 2 cos(w d_k)
            _, _, dk_dr2 = _stationary_parts(b, t1, t2)
            dp = dk_dr2 * (-2.0 * w * S)
        elif b.kind == "nn":  # A = s0 + sigma^2 sum_k cos(w d_k); B, C do not depend on w
            _, _, _, q, u, _ = _nn_parts(b, t1, t2)
            dp = b.magn ** 2 * (2.0 / math.pi) / np.sqrt(1 - u * u) * (2.0 * b.sigma ** 2 * w * S / q)
        else:
            raise ValueError(b.kind)
        return K, [dp] + gb
    grads = {}
    if cf.kind == "const":
        K = np.full((n1, n2), cf.magn ** 2)
    elif cf.kind == "lin":
        K = cf.magn ** 2 * (x1 @ x2.T)
    elif cf.kind in _STATIONARY:
        K, grads["lscale"], _ = _stationary_parts(cf, x1, x2)
    elif cf.kind == "nn":
        A, B, Cc, q, u, K = _nn_parts(cf, x1, x2)
        dk_du = cf.magn ** 2 * (2.0 / math.pi) / np.sqrt(1 - u * u)
        s0 = cf.sigma0 ** 2 * cf.sigma ** 2
        # dlog(sigma0): dA = dB = dC = 2 s0; dlog(sigma): dA = 2A, dB = 2B, dC = 2C
        grads["sigma0"] = dk_du * (4 * s0 / q - u * (2 * s0 / (1 + 2 * B) + 2 * s0 / (1 + 2 * Cc)))
        grads["sigma"] = dk_du * (4 * A / q - u * (2 * B / (1 + 2 * B) + 2 * Cc / (1 + 2 * Cc)))
    else:
        raise ValueError(cf.kind)
    grads["magn"] = 2.0 * K
    return K, [grads[nm] for nm in PARAM_NAMES[cf.kind] if not _is_fixed(cf, nm)]


def kernel_grads_complex_step(cfs, x1, x2, h=1e-20):
    """dK/dlog(theta) of eval_cf.list for every free covariance parameter (get_param
    order) by complex-step differentiation of eval_cf: the independent pin of
    kernel_and_grads."""
    import cmath
    import copy
    vals = []
    for cf in cfs:
        vals += get_param_cf(cf)[1]
    out = []
    for j in range(len(vals)):
        cc = copy.deepcopy(cfs)
        v = np.array(vals, dtype=np.complex128)
        v[j] += 1j * h
        k = 0
        for cf in cc:
            k += _set_param_cf(cf, v[k:], exp=cmath.exp)
        out.append(np.imag(eval_cf(cc, x1, x2)) / h)
    return out


def dlpdf_prior(gp):
    """Derivative of lpdf_prior (R/priors.R:96-112) with respect to the log-parameters."""
    def one(prior, param):
        if prior is None or prior.kind in ("fixed", "logunif"):
            return 0.0
        if prior.kind == "lognormal":
            return -(param - prior.loc) / prior.scale ** 2
        if prior.kind == "half_t":
            t = math.exp(param) / prior.scale
            return 1.0 - (prior.df + 1) * t * t / (prior.df + t * t)
        raise ValueError(prior.kind)

    def cf_terms(cf):
        if cf.kind == "prod":
            return sum((cf_terms(c) for c in cf.cfs), [])
        if cf.kind == "periodic":
            t = [] if _is_fixed(cf, "period") else [one(cf.priors.get("period"), math.log(cf.period))]
            return t + cf_terms(cf.base)
        return [one(cf.priors.get(nm), math.log(getattr(cf, nm)))
                for nm in PARAM_NAMES[cf.kind] if not _is_fixed(cf, nm)]
    g = sum((cf_terms(cf) for cf in gp.cfs), [])
    g += [one(gp.lik.priors.get(nm), math.log(getattr(gp.lik, nm)))
          for nm in PARAM_NAMES[gp.lik.kind] if not _is_fixed(gp.lik, nm)]
    return np.array(g, dtype=np.float64)


def log_evidence_grad(gp, threads=1, block=1024):
    """d log_evidence / d log(theta) of a fitted lik_gaussian + method_full GP, for the
    free parameters in get_param order: (1/2) sum_ij W_ij dK_ij per covariance
    parameter, W = alpha alpha^T - C^-1, and sigma^2 (alpha^T alpha - tr C^-1) for
    the noise. Row blocks of W and dK are formed one at a time (threads of them in
    parallel); their sums are added in block order."""
    from scipy.linalg import lapack
    if gp.lik.kind != "gaussian" or gp.method.kind != "full":
        raise ValueError("the gradient is defined for lik_gaussian with method_full")
    x = gp.x
    n = x.shape[0]
    alpha = gp.fit["alpha"]
    Ci, info = lapack.dpotri(gp.fit["C_chol"], lower=1)
    if info != 0:
        raise np.linalg.LinAlgError("potri failed")
    il = np.tril_indices(n, -1)
    Ci[il[1], il[0]] = Ci[il]  # symmetric fill from the lower triangle
    bounds = list(range(0, n, block)) + [n]

    def part(b):
        i0, i1 = b
        grads = []
        for cf in gp.cfs:
            grads += kernel_and_grads(cf, x[i0:i1], x)[1]
        Wb = alpha[i0:i1, None] * alpha[None, :] - Ci[i0:i1]
        return np.array([(Wb * g).sum() for g in grads])
    blocks = list(zip(bounds[:-1], bounds[1:]))
    if threads > 1:
        from concurrent.futures import ThreadPoolExecutor
        with ThreadPoolExecutor(threads) as ex:
            parts = list(ex.map(part, blocks))
    else:
        parts = [part(b) for b in blocks]
    g = 0.5 * np.sum(parts, axis=0) if parts and len(parts[0]) else np.zeros(0)
    g = list(g)
    for nm in PARAM_NAMES[gp.lik.kind]:
        if not _is_fixed(gp.lik, nm):
            s2 = gp.lik.sigma ** 2
            g.append(s2 * (alpha @ alpha - np.trace(Ci)))
    return np.array(g, dtype=np.float64)


def gp_energy_grad(gp, include_prior=True, threads=1):
    """Gradient of gp_energy (R/gp.R:138-147) with respect to the log-parameters."""
    g = -log_evidence_grad(gp, threads=threads)
    if include_prior:
        g = g - dlpdf_prior(gp)
    return g


def gp_pred_post_full(gp, xt, var=False, cfind=None):
    """gp_pred_post.method_full (R/gp_pred.R:202-232)."""
    Kt = eval_cf(gp.cfs, xt, gp.x, cfind)
    mean = Kt @ gp.fit["alpha"]
    if not var:
        return dict(mean=mean)
    Ktt_diag = eval_cf(gp.cfs, xt, xt, cfind, diag_only=True)
    if gp.fit.get("C_chol") is None:  # LU of K + diag(V) (non-log-concave fit, R/gp_pred.R:220-223)
        return dict(mean=mean, var=Ktt_diag - (Kt * sla.lu_solve(gp.fit["C_lu"], Kt.T).T).sum(1))
    aux = sla.solve_triangular(gp.fit["C_chol"], Kt.T, lower=True)
    return dict(mean=mean, var=Ktt_diag - (aux * aux).sum(0))


def gp_pred_post_fitc(gp, xt, var=False, train=False, cfind=None):
    """gp_pred_post.method_fitc (R/gp_pred.R:234-296), var (not cov) branch."""
    z = as_matrix(gp.method.inducing)
    alpha = gp.fit["alpha"]
    Ktz = eval_cf(gp.cfs, xt, z, cfind)
    Kxz = gp.fit["Kxz"]
    Kz_chol = gp.fit["Kz_chol"]
    Dt = None
    if var or train:
        Dt = eval_cf(gp.cfs, xt, xt, cfind, diag_only=True)
        Dt = Dt - (sla.solve_triangular(Kz_chol, Ktz.T, lower=True) ** 2).sum(0)
    A1 = sla.solve_triangular(Kz_chol, Kxz.T, lower=True)
    A2 = sla.solve_triangular(Kz_chol, Ktz.T, lower=True)
    mean = A2.T @ (A1 @ alpha)
    if train:
        mean = mean + Dt * alpha
    if not var:
        return dict(mean=mean)
    Ci = gp.fit["C_inv"]
    Kz_inv_Ktz = _chol_solve_lower(Kz_chol, Ktz.T)
    prior_var = (Ktz * Kz_inv_Ktz.T).sum(1) + Dt
    if train:
        aux = inv_lemma_solve(Ci, A1.T, A1) @ A2 + inv_lemma_solve(Ci, Dt, A1, rhs_diag=True)
        d1 = (A2 * aux).sum(0)
        d2 = (inv_lemma_solve(Ci, A1.T, Dt, lhs_diag=True) * A2.T).sum(1)
        d3 = inv_lemma_solve(Ci, Dt, Dt, rhs_diag=True, lhs_diag=True, diag_only=True)
        red = d1 + d2 + d3
    else:
        aux = inv_lemma_solve(Ci, A1.T, A1) @ A2
        red = (A2 * aux).sum(0)
    return dict(mean=mean, var=prior_var - red)


def gp_pred(gp, xnew, var=False, quantiles=None, transform=False, cfind=None, quad_order=15,
            offset=None):
    """gp_pred (R/gp_pred.R:88-122) for fitted models; prior prediction (R/gp_pred.R:142-156)
    when not fitted (full method)."""
    xnew = as_matrix(xnew)
    if quantiles is not None or transform:
        var = True
    if getattr(gp, "fit", None) is None:
        mean = np.zeros(xnew.shape[0])
        pred = dict(mean=mean)
        if var and gp.method.kind in ("rf", "rbf"):
            zt = get_featuremap(gp, xnew.shape[1])(xnew, cfind)  # R/gp_pred.R:186-200
            pred["var"] = (zt * zt).sum(1)
        elif var:
            pred["var"] = eval_cf(gp.cfs, xnew, xnew, cfind, diag_only=True)
    else:
        if not gp.fitted:
            raise RuntimeError("The GP object seems to contain a posterior fit, but is not refitted")
        if gp.method.kind == "full":
            pred = gp_pred_post_full(gp, xnew, var, cfind)
        elif gp.method.kind in ("rf", "rbf"):
            pred = gp_pred_post_rf(gp, xnew, var, cfind)
        else:
            pred = gp_pred_post_fitc(gp, xnew, var, False, cfind)
    pred["mean"] = add_offset(pred["mean"], offset)
    if quantiles is not None:
        from scipy.stats import norm
        q = np.stack([norm.ppf(qq, loc=pred["mean"], scale=np.sqrt(pred["var"])) for qq in quantiles], 1)
        if transform:
            q = get_response(gp.lik, q)
        pred["quantiles"] = q
    if transform:
        fg, w = gauss_hermite_points_scaled(pred["mean"], np.sqrt(pred["var"]), quad_order)
        ft = get_response(gp.lik, fg)
        mt = ft @ w
        pred["mean"] = mt
        pred["var"] = ((ft - mt[:, None]) ** 2) @ w
    return pred


def loo_posteriors(gp, x):
    """loo_posteriors.approx_laplace / .approx_ep (R/gp_loo.R:119-133)."""
    fit = gp.fit
    if gp.approx.kind == "ep":
        return fit["cavity_mean"], fit["cavity_var"]
    fhat = np.asarray(fit["fmean"]).ravel()
    z, V = fit["z"], fit["V"]
    grad = (z - fhat) / V
    if gp.method.kind == "full":
        pv = gp_pred_post_full(gp, as_matrix(x), var=True)["var"]
    elif gp.method.kind in ("rf", "rbf"):
        pv = gp_pred_post_rf(gp, as_matrix(x), var=True)["var"]
    else:
        pv = gp_pred_post_fitc(gp, as_matrix(x), var=True, train=True)["var"]
    loo_var = 1 / (1 / pv - 1 / V)
    return fhat - loo_var * grad, loo_var


def gp_loo(gp, x, y, quad_order=11, trials=None, offset=None, z=None):
    """gp_loo (R/gp_loo.R:73-109): the quadrature branch, or with z (n x draws standard
    normals standing in for stats::rnorm's, filled in R's column-major order) the Monte
    Carlo branch: fsample = loo_mean + sqrt(loo_var) z, loos = logsumexp - log(draws)."""
    if getattr(gp, "fit", None) is None or not gp.fitted:
        raise RuntimeError("The provided GP model is not fitted.")
    m, v = loo_posteriors(gp, x)
    if z is not None:
        fs = m[:, None] + np.sqrt(v)[:, None] * z
        ll = get_loglik(gp.lik, fs, y, trials, offset, sum_=False)
        loos = logsumexp_rows(ll) - math.log(z.shape[1])
    else:
        fg, w = gauss_hermite_points_scaled(m, np.sqrt(v), quad_order)
        ll = get_loglik(gp.lik, fg, y, trials, offset, sum_=False)
        loos = logsumexp_rows(ll, w)
    n = len(y)
    return dict(loo=float(loos.sum()), sd=float(n * (np.std(loos, ddof=1) / math.sqrt(n))), loos=loos)


# ----------------------------------------------------------------------------
# Constructors (R/cf.R:88-195, R/lik.R:44-90, R/method.R:105-125, R/approx.R:60-75,
# R/priors.R:56-91, R/gp.R:52-71) -- plain namespaces for the oracle's own tests
# ----------------------------------------------------------------------------

def prior(kind, **kw):
    return SimpleNamespace(kind=kind, **kw)


def cf(kind, vars=None, normalize=False, priors=None, **params):
    defaults = dict(const=dict(magn=1.0), lin=dict(magn=1.0), sexp=dict(lscale=0.3, magn=1.0),
                    matern32=dict(lscale=0.3, magn=1.0), matern52=dict(lscale=0.3, magn=1.0),
                    nn=dict(sigma0=1.0, sigma=3.0, magn=1.0), periodic=dict(period=1.0))[kind]
    defaults.update(params)
    o = SimpleNamespace(kind=kind, vars=vars, normalize=normalize, means=None, scales=None,
                        priors=priors or {}, **defaults)
    if kind == "nn" and "normalize" not in params and normalize is False:
        pass
    if kind == "periodic" and not hasattr(o, "base"):
        o.base = cf("sexp")
    return o


def cf_periodic(period=1.0, base=None, vars=None, priors=None):
    b = base if base is not None else cf("sexp")
    b.normalize = False
    b.vars = None
    return SimpleNamespace(kind="periodic", vars=vars, normalize=False, means=None, scales=None,
                           priors=priors or {}, period=period, base=b)


def cf_prod(*cfs):
    flat = []
    for c in cfs:
        flat += c.cfs if c.kind == "prod" else [c]
    return SimpleNamespace(kind="prod", cfs=flat, vars=None, normalize=False, priors={})


def lik(kind, link=None, priors=None, **params):
    defaults = dict(gaussian=dict(sigma=0.5), bernoulli={}, binomial={}, betabinom=dict(phi=1.0),
                    poisson={})[kind]
    defaults.update(params)
    dl = dict(gaussian="identity", bernoulli="logit", binomial="logit", betabinom="logit",
              poisson="log")[kind]
    return SimpleNamespace(kind=kind, link=link or dl, priors=priors or {}, **defaults)


def method_full():
    return SimpleNamespace(kind="full")


def method_fitc(inducing):
    inducing = as_matrix(inducing)
    return SimpleNamespace(kind="fitc", inducing=inducing, num_inducing=inducing.shape[0])


def approx_laplace(maxiter=30, tol=1e-4):
    return SimpleNamespace(kind="laplace", maxiter=maxiter, tol=tol)


def approx_ep(damping=0.9, quad_order=11, maxiter=100):
    return SimpleNamespace(kind="ep", damping=damping, quad_order=quad_order, maxiter=maxiter)


def gp_init(cfs, lik_, method=None, approx=None):
    if not isinstance(cfs, (list, tuple)):
        cfs = [cfs]
    approx = approx or approx_laplace()
    if approx.kind == "ep" and lik_.kind == "gaussian":
        raise ValueError("approx_ep disabled for lik_gaussian")
    method = method or method_full()
    if method.kind in ("rf", "rbf"):
        method.num_basis = check_num_basis(cfs, method.num_basis)  # R/gp.R:64-66
    return SimpleNamespace(cfs=list(cfs), lik=lik_, method=method, approx=approx,
                           fitted=False, fit=None, x=None)
