"""Model objects of gplite: covariance functions, likelihoods, methods,
approximations and priors, with the reference's constructors, defaults,
parameter names and log-space get/set semantics.

Constructors: R/cf.R:92-213, R/lik.R:44-90, R/method.R:105-125,
R/approx.R:60-75, R/priors.R:56-91. Parameter handling: R/cf.R:283-396,
R/lik.R:118-168, R/misc.R:33-56. Input columns ``vars`` are 0-based indices
(the reference takes 1-based indices or column names).
"""
from __future__ import annotations

import copy
import math
import warnings

import numpy as np

# ----------------------------------------------------------------------------
# priors (R/priors.R)
# ----------------------------------------------------------------------------


class Prior:
    kind = "prior"

    def lpdf(self, param: float) -> float:  # log density of the log-parameter
        return 0.0

    def dlpdf(self, param: float) -> float:
        return 0.0

    def __repr__(self):
        return "prior_%s()" % self.kind


class prior_fixed(Prior):
    kind = "fixed"


class prior_logunif(Prior):
    kind = "logunif"


class prior_lognormal(Prior):
    kind = "lognormal"

    def __init__(self, loc=0.0, scale=1.0):
        self.loc, self.scale = float(loc), float(scale)

    def lpdf(self, param):  # stats::dnorm(param, loc, scale, log = TRUE) (R/priors.R:110-112)
        return -0.5 * math.log(2 * math.pi) - math.log(self.scale) - 0.5 * ((param - self.loc) / self.scale) ** 2

    def dlpdf(self, param):
        return -(param - self.loc) / self.scale ** 2


class prior_half_t(Prior):
    kind = "half_t"

    def __init__(self, df=1.0, scale=1.0):
        self.df, self.scale = float(df), float(scale)

    def lpdf(self, param):  # R/priors.R:102-107
        df, sc = self.df, self.scale
        t = math.exp(param) / sc
        ldt = (math.lgamma((df + 1) / 2) - math.lgamma(df / 2) - 0.5 * math.log(df * math.pi)
               - (df + 1) / 2 * math.log1p(t * t / df))
        return math.log(2) - math.log(sc) + ldt + param

    def dlpdf(self, param):
        t = math.exp(param) / self.scale
        return 1.0 - (self.df + 1) * t * t / (self.df + t * t)


# ----------------------------------------------------------------------------
# covariance functions (R/cf.R)
# ----------------------------------------------------------------------------

PARAM_NAMES = {
    "const": ["magn"], "lin": ["magn"], "sexp": ["lscale", "magn"],
    "matern32": ["lscale", "magn"], "matern52": ["lscale", "magn"],
    "nn": ["sigma0", "sigma", "magn"], "periodic": ["period"],
}
# gradient slot of each parameter in the C ABI (lscale, magn, sigma0, sigma, period)
GRAD_SLOT = {"lscale": 0, "magn": 1, "sigma0": 2, "sigma": 3, "period": 4}


class Cf:
    kind = "cf"

    def __init__(self, vars=None, normalize=False, priors=None, **params):
        self.vars = None if vars is None else [int(v) for v in np.atleast_1d(vars)]
        self.normalize = bool(normalize)
        self.means = None
        self.scales = None
        self.priors = dict(priors or {})
        for k, v in params.items():
            setattr(self, k, float(v))

    @property
    def name(self):
        return "cf_" + self.kind

    def __mul__(self, other):  # "*.cf" (R/cf.R:199-213)
        return cf_prod(self, other)

    def is_fixed(self, pname):
        p = self.priors.get(pname)
        return p is not None and p.kind == "fixed"

    def param_names(self):
        return [n for n in PARAM_NAMES[self.kind] if not self.is_fixed(n)]

    def get_param(self):
        names = self.param_names()
        return [self.name + "." + n for n in names], [math.log(getattr(self, n)) for n in names]

    def set_param(self, vals):
        names = self.param_names()
        for n, v in zip(names, vals):
            setattr(self, n, math.exp(v))
        return len(names)

    def lpdf_prior(self):
        return sum(self.priors.get(n, prior_logunif()).lpdf(math.log(getattr(self, n)))
                   for n in self.param_names())

    def dlpdf_prior(self):
        return [self.priors.get(n, prior_logunif()).dlpdf(math.log(getattr(self, n)))
                for n in self.param_names()]

    def learn_scales(self, x):  # learn_scales.cf (R/cf.R:836-845)
        xs = x if self.vars is None else x[:, self.vars]
        self.means = xs.mean(axis=0)
        self.scales = xs.std(axis=0, ddof=1)

    def __repr__(self):
        ps = "; ".join("%s = %.3g" % (n, getattr(self, n)) for n in PARAM_NAMES[self.kind])
        v = "" if self.vars is None else "vars = %s; " % ",".join(map(str, self.vars))
        return "%s(%s%s)" % (self.name, v, ps)


def cf_const(magn=1.0, prior_magn=None):
    c = Cf(priors={"magn": prior_magn or prior_logunif()}, magn=magn)
    c.kind = "const"
    return c


def _cf(kind, vars, normalize, **kw):
    c = Cf(vars=vars, normalize=normalize, **kw)
    c.kind = kind
    return c


def cf_lin(vars=None, magn=1.0, prior_magn=None, normalize=False):
    return _cf("lin", vars, normalize, priors={"magn": prior_magn or prior_logunif()}, magn=magn)


def cf_sexp(vars=None, lscale=0.3, magn=1.0, prior_lscale=None, prior_magn=None, normalize=False):
    return _cf("sexp", vars, normalize,
               priors={"lscale": prior_lscale or prior_logunif(), "magn": prior_magn or prior_logunif()},
               lscale=lscale, magn=magn)


def cf_matern32(vars=None, lscale=0.3, magn=1.0, prior_lscale=None, prior_magn=None, normalize=False):
    return _cf("matern32", vars, normalize,
               priors={"lscale": prior_lscale or prior_logunif(), "magn": prior_magn or prior_logunif()},
               lscale=lscale, magn=magn)


def cf_matern52(vars=None, lscale=0.3, magn=1.0, prior_lscale=None, prior_magn=None, normalize=False):
    return _cf("matern52", vars, normalize,
               priors={"lscale": prior_lscale or prior_logunif(), "magn": prior_magn or prior_logunif()},
               lscale=lscale, magn=magn)


def cf_nn(vars=None, sigma0=1.0, sigma=3.0, magn=1.0, prior_sigma0=None, prior_sigma=None,
          prior_magn=None, normalize=True):
    return _cf("nn", vars, normalize,
               priors={"sigma0": prior_sigma0 or prior_half_t(), "sigma": prior_sigma or prior_half_t(),
                       "magn": prior_magn or prior_logunif()},
               sigma0=sigma0, sigma=sigma, magn=magn)


class CfPeriodic(Cf):
    kind = "periodic"

    def __init__(self, vars=None, period=1.0, cf_base=None, prior_period=None):
        super().__init__(vars=vars, normalize=False, priors={"period": prior_period or prior_logunif()},
                         period=period)
        base = copy.deepcopy(cf_base) if cf_base is not None else cf_sexp()
        if base.kind in ("periodic", "prod"):
            raise ValueError("cf_periodic base must be a plain covariance function")
        base.normalize = False  # R/cf.R:181-182
        base.vars = None
        self.base = base

    def get_param(self):  # get_param.cf_periodic (R/cf.R:325-334)
        names, vals = self.base.get_param()
        names = ["cf_periodic." + s.split(".", 1)[1] for s in names]
        if not self.is_fixed("period"):
            names = ["cf_periodic.period"] + names
            vals = [math.log(self.period)] + vals
        return names, vals

    def set_param(self, vals):
        j = 0
        if not self.is_fixed("period"):
            self.period = math.exp(vals[0])
            j = 1
        return j + self.base.set_param(vals[j:])

    def lpdf_prior(self):
        lp = 0.0 if self.is_fixed("period") else self.priors["period"].lpdf(math.log(self.period))
        return lp + self.base.lpdf_prior()

    def dlpdf_prior(self):
        d = [] if self.is_fixed("period") else [self.priors["period"].dlpdf(math.log(self.period))]
        return d + self.base.dlpdf_prior()

    def learn_scales(self, x):  # periodic cf does not normalise (R/cf.R:852-855)
        pass


def cf_periodic(vars=None, period=1.0, cf_base=None, prior_period=None):
    return CfPeriodic(vars=vars, period=period, cf_base=cf_base, prior_period=prior_period)


class CfProd(Cf):
    kind = "prod"

    def __init__(self, *cfs):
        super().__init__()
        flat = []
        for c in cfs:
            flat += list(c.cfs) if c.kind == "prod" else [copy.deepcopy(c)]
        self.cfs = flat
        names, _ = self.get_param()
        if sum("magn" in n for n in names) > 1:  # R/misc.R:67-100
            warnings.warn("Detected a product of covariance functions with more than one non-fixed "
                          "magnitude parameters.")

    def get_param(self):
        names, vals = [], []
        for c in self.cfs:
            n_, v_ = c.get_param()
            names += n_
            vals += v_
        return names, vals

    def set_param(self, vals):
        j = 0
        for c in self.cfs:
            j += c.set_param(vals[j:])
        return j

    def lpdf_prior(self):
        return sum(c.lpdf_prior() for c in self.cfs)

    def dlpdf_prior(self):
        out = []
        for c in self.cfs:
            out += c.dlpdf_prior()
        return out

    def learn_scales(self, x):
        for c in self.cfs:
            c.learn_scales(x)

    def __repr__(self):
        return "cf_prod(" + ", ".join(repr(c) for c in self.cfs) + ")"


def cf_prod(*cfs):
    return CfProd(*cfs)


# ----------------------------------------------------------------------------
# likelihoods (R/lik.R)
# ----------------------------------------------------------------------------

LIK_PARAMS = {"gaussian": ["sigma"], "bernoulli": [], "binomial": [], "betabinom": ["phi"], "poisson": []}


class LikObj:
    def __init__(self, kind, link, priors=None, **params):
        self.kind = kind
        self.link = link
        self.priors = dict(priors or {})
        for k, v in params.items():
            setattr(self, k, float(v))

    @property
    def name(self):
        return "lik_" + self.kind

    def is_fixed(self, pname):
        p = self.priors.get(pname)
        return p is not None and p.kind == "fixed"

    def param_names(self):
        return [n for n in LIK_PARAMS[self.kind] if not self.is_fixed(n)]

    def get_param(self):
        names = self.param_names()
        return [self.name + "." + n for n in names], [math.log(getattr(self, n)) for n in names]

    def set_param(self, vals):
        names = self.param_names()
        for n, v in zip(names, vals):
            setattr(self, n, math.exp(v))
        return len(names)

    def lpdf_prior(self):
        return sum(self.priors.get(n, prior_logunif()).lpdf(math.log(getattr(self, n)))
                   for n in self.param_names())

    def dlpdf_prior(self):
        return [self.priors.get(n, prior_logunif()).dlpdf(math.log(getattr(self, n)))
                for n in self.param_names()]

    def response(self, f):  # get_response.lik_* (R/lik.R:460-498)
        f = np.asarray(f, dtype=np.float64)
        if self.kind == "gaussian":
            return f
        if self.kind == "poisson":
            return np.exp(f)
        if self.link == "probit":
            from scipy.special import ndtr
            return ndtr(f)
        return 1 / (1 + np.exp(-f))

    def __repr__(self):
        ps = "; ".join("%s = %.3g" % (n, getattr(self, n)) for n in LIK_PARAMS[self.kind])
        return "%s(%s)" % (self.name, ps)


def lik_gaussian(sigma=0.5, prior_sigma=None):
    return LikObj("gaussian", "identity", priors={"sigma": prior_sigma or prior_logunif()}, sigma=sigma)


def lik_bernoulli(link="logit"):
    return LikObj("bernoulli", link)


def lik_binomial(link="logit"):
    return LikObj("binomial", link)


def lik_betabinom(link="logit", phi=1.0, prior_phi=None):
    return LikObj("betabinom", link, priors={"phi": prior_phi or prior_logunif()}, phi=phi)


def lik_poisson(link="log"):
    return LikObj("poisson", link)


# ----------------------------------------------------------------------------
# methods and approximations (R/method.R:105-125, R/approx.R:60-75)
# ----------------------------------------------------------------------------


class MethodObj:
    def __init__(self, kind, **kw):
        self.kind = kind
        for k, v in kw.items():
            setattr(self, k, v)

    def __repr__(self):
        return "method_" + self.kind


def method_full():
    return MethodObj("full")


def method_fitc(inducing=None, num_inducing=100, bin_along=None, bin_count=10, seed=12345):
    if inducing is not None:
        inducing = np.asarray(inducing, dtype=np.float64)
        if inducing.ndim == 1:
            inducing = inducing[:, None]
        num_inducing = inducing.shape[0]
    return MethodObj("fitc", inducing=inducing, num_inducing=int(num_inducing), bin_along=bin_along,
                     bin_count=min(bin_count, num_inducing), seed=seed)


def method_rf(num_basis=400, seed=12345):
    """method_rf (R/method.R:129-133): random features (a linearised GP with num_basis
    features per covariance function, drawn from the seed)."""
    return MethodObj("rf", num_basis=num_basis, seed=seed)


def method_rbf(num_basis=400, seed=12345):
    """method_rbf (R/method.R:135-139): radial basis features centred at num_basis
    training inputs drawn from the seed."""
    return MethodObj("rbf", num_basis=num_basis, seed=seed)


class ApproxObj:
    def __init__(self, kind, **kw):
        self.kind = kind
        for k, v in kw.items():
            setattr(self, k, v)

    def __repr__(self):
        return "approx_" + self.kind


def approx_laplace(maxiter=30, tol=1e-4):
    return ApproxObj("laplace", maxiter=int(maxiter), tol=float(tol))


def approx_ep(damping=0.9, quad_order=11, maxiter=100):
    if damping <= 0 or damping >= 1:
        raise ValueError("Damping should be between 0 and 1 (exclusive)")
    return ApproxObj("ep", damping=float(damping), quad_order=int(quad_order), maxiter=int(maxiter))
