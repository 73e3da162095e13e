"""gplite's user API on top of libgpgp: gp_init, gp_fit, gp_energy, gp_pred,
gp_loo, gp_compare, gp_optim, get_param / set_param.

Same names, argument meanings, defaults and error behaviour as the R package
(R/gp.R:52-205, R/gp_fit.R:54-60, R/gp_pred.R:88-122, R/gp_loo.R:73-175,
R/gp_optim.R:63-160); the numerical work of fit / pred / LOO runs in the CUDA
library through the C ABI (include/gpgp.h). Only O(p) host logic (parameter
packing, priors, learn_scales, the optimiser loop) runs in Python.
"""
from __future__ import annotations

import ctypes as C
import math
import warnings

import numpy as np

from . import _lib as L
from .objects import (GRAD_SLOT, Cf, approx_ep, approx_laplace, cf_sexp, lik_gaussian,
                      method_full)

RF_METHODS = ("rf", "rbf")

JITTER_DEFAULT = 1e-6  # get_jitter (R/gp.R:276-281)


class GP:
    """A GP model (the reference's list of class "gp", R/gp.R:57-69)."""

    def __init__(self, cfs, lik, method, approx):
        self.cfs = cfs
        self.lik = lik
        self.method = method
        self.approx = approx
        self.fitted = False
        self.fit = None
        self.x = None
        self._model = None

    def __del__(self):
        self._free()

    def _free(self):
        m = getattr(self, "_model", None)
        if m:
            try:
                L.load().gpgp_model_free(m)
            except Exception:
                pass
        self._model = None

    def __repr__(self):
        return ("Likelihood:\n  %r\nCovariance functions:\n%s\nMethod:\n  %r\nLatent approximation:\n  %r"
                % (self.lik, "\n".join("  %r" % c for c in self.cfs), self.method, self.approx))


def gp_init(cfs=None, lik=None, method=None, approx=None) -> GP:
    """gp_init (R/gp.R:52-71)."""
    cfs = cf_sexp() if cfs is None else cfs
    lik = lik_gaussian() if lik is None else lik
    method = method_full() if method is None else method
    approx = approx_laplace() if approx is None else approx
    if lik.kind == "gaussian" and approx.kind == "ep":
        raise ValueError("approx_ep disabled for lik_gaussian: use approx_laplace instead, because it "
                         "gives exact results")
    if isinstance(cfs, Cf):
        cfs = [cfs]
    if method.kind in RF_METHODS:
        method.num_basis = check_num_basis(cfs, method.num_basis)  # R/gp.R:64-66
    return GP(list(cfs), lik, method, approx)


def check_num_basis(cfs, num_basis, num_inputs=None):
    """check_num_basis (R/gp.R:211-233): one count per covariance function; cf_const takes
    1 feature and cf_lin its number of inputs (None while that is unknown, R's NA)."""
    if num_basis is None:
        return None
    nb = [None if v is None else int(v) for v in np.atleast_1d(np.asarray(num_basis, dtype=object))]
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


def _rf_term_inputs(c, d):
    """Input columns a term's feature map reads: its vars (all d when unset), twice
    that under cf_periodic (sin and cos, R/cf.R:659-674)."""
    nv = len(c.vars) if c.vars is not None else d
    return 2 * nv if c.kind == "periodic" else nv


def _rf_draws(gp, d, x=None):
    """The random draws of the feature maps (rf_featmap / rbf_featmap, R/cf.R:571-817), one
    array per device term (None for cf_const / cf_lin) in the layout include/gpgp.h gives.
    Every covariance function (and every factor of a product) starts from the method's seed,
    as the reference calls set.seed(seed) in each feature-map constructor; numpy's generator
    stands in for R's stream (the same shapes and distributions, other numbers). rbf centres
    are training inputs sampled without replacement (R's sample(n, num_feat))."""
    me = gp.method
    nb = check_num_basis(gp.cfs, me.num_basis, d)
    out = []
    for g, c in _flat_terms(gp):
        base = c.base if c.kind == "periodic" else c
        q = _rf_term_inputs(c, d)
        rng = np.random.default_rng(me.seed)
        if base.kind in ("const", "lin"):
            out.append(None)
            continue
        if base.kind in ("matern32", "matern52"):
            raise ValueError("Random Fourier features for Matern kernels not implemented yet." if me.kind == "rf"
                             else "RBF features are not available for Matern kernels")
        if me.kind == "rf":
            if base.kind == "sexp":
                if nb[g] % 2 == 1:
                    raise ValueError("number of features must be an even number.")
                out.append(rng.standard_normal((nb[g] // 2) * q))  # matrix(rnorm(m q), nrow = q)
            else:  # nn: w (q x m), then w0 (m)
                w = rng.standard_normal(nb[g] * q)
                out.append(np.concatenate([w, rng.standard_normal(nb[g])]))
        else:
            if base.kind != "sexp":
                raise ValueError("RBF features are not available for cf_%s" % base.kind)
            if x is None:
                raise RuntimeError("Cannot compute RBF feature map when the x matrix is not known.")
            xs = x if c.vars is None else x[:, c.vars]
            if c.kind == "periodic":
                w = 2 * math.pi / c.period
                xs = np.hstack([np.sin(w * xs), np.cos(w * xs)])
            if nb[g] > xs.shape[0]:
                raise ValueError("cannot take a sample larger than the population when 'replace = FALSE'")
            ind = rng.choice(xs.shape[0], nb[g], replace=False)
            out.append(np.ascontiguousarray(xs[ind]).ravel())  # column j of q x nb = centre j
    return nb, out


def _method_struct(gp, d, x=None):
    """The C method struct; for rf / rbf also the arrays its pointers refer to (kept by
    the caller for the duration of the call)."""
    me = L.Method()
    me.kind = L.METHOD[gp.method.kind]
    keep = []
    if gp.method.kind in RF_METHODS:
        nb, draws = _rf_draws(gp, d, x)
        for g, v in enumerate(nb):
            me.num_basis[g] = int(v)
        for t, a in enumerate(draws):
            if a is not None:
                a = np.ascontiguousarray(a, dtype=np.float64)
                keep.append(a)
                me.draws[t] = a.ctypes.data
    return me, keep


# ----------------------------------------------------------------------------
# parameters (R/gp.R:149-169)
# ----------------------------------------------------------------------------

def get_param(gp):
    """get_param.gp: log-parameters, cfs in order then the likelihood; returns (names, values)."""
    names, vals = [], []
    for c in gp.cfs:
        n_, v_ = c.get_param()
        names += n_
        vals += v_
    n_, v_ = gp.lik.get_param()
    return names + n_, np.array(vals + v_, dtype=np.float64)


def set_param(gp, param):
    """set_param.gp: sets log-parameters and marks the model as needing a refit."""
    param = list(np.asarray(param, dtype=np.float64).ravel())
    j = 0
    for c in gp.cfs:
        j += c.set_param(param[j:])
    j += gp.lik.set_param(param[j:])
    if j != len(param):
        raise ValueError("expected %d parameters, got %d" % (j, len(param)))
    gp.fitted = False
    return gp


def lpdf_prior(gp):
    return sum(c.lpdf_prior() for c in gp.cfs) + gp.lik.lpdf_prior()


def _dlpdf_prior(gp):
    out = []
    for c in gp.cfs:
        out += c.dlpdf_prior()
    return np.array(out + gp.lik.dlpdf_prior(), dtype=np.float64)


# ----------------------------------------------------------------------------
# translation to the C ABI
# ----------------------------------------------------------------------------

def _flat_terms(gp):
    """(group, cf) for every device term, in parameter order."""
    out = []
    for g, c in enumerate(gp.cfs):
        for t in (c.cfs if c.kind == "prod" else [c]):
            out.append((g, t))
    return out


def _fill_term(T, g, c, d):
    T.group = g
    periodic = c.kind == "periodic"
    base = c.base if periodic else c
    T.kind = L.CF_KIND[base.kind]
    T.periodic = 1 if periodic else 0
    T.normalize = 1 if (getattr(c, "normalize", False) and c.means is not None and not periodic) else 0
    if c.vars is not None:
        if len(c.vars) > L.MAX_VARS:
            raise ValueError("too many vars in one covariance function")
        T.nvars = len(c.vars)
        for i, v in enumerate(c.vars):
            if not 0 <= v < d:
                raise ValueError("vars index %d out of range for d = %d" % (v, d))
            T.vars[i] = v
    else:
        T.nvars = 0
    if T.normalize:
        for i, (mu, sd) in enumerate(zip(np.atleast_1d(c.means), np.atleast_1d(c.scales))):
            T.means[i] = mu
            T.scales[i] = sd
    T.lscale = getattr(base, "lscale", 1.0)
    T.magn = getattr(base, "magn", 1.0)
    T.sigma0 = getattr(base, "sigma0", 0.0)
    T.sigma = getattr(base, "sigma", 0.0)
    T.period = getattr(c, "period", 1.0)


def kernel_struct(cfs, d):
    gp = GP(cfs, None, None, None)
    terms = _flat_terms(gp)
    if len(terms) > L.MAX_TERMS:
        raise ValueError("at most %d covariance terms are supported" % L.MAX_TERMS)
    k = L.Kernel()
    k.nterms = len(terms)
    k.ngroups = len(cfs)
    for i, (g, c) in enumerate(terms):
        _fill_term(k.term[i], g, c, d)
    return k


def _lik_struct(lik):
    s = L.Lik()
    s.kind = L.LIK_KIND[lik.kind]
    s.link = L.LINK[lik.link]
    s.sigma = getattr(lik, "sigma", 0.0)
    s.phi = getattr(lik, "phi", 0.0)
    return s


def _approx_struct(gp):
    a = L.Approx()
    ap = gp.approx
    a.kind = L.APPROX[ap.kind]
    a.maxiter = ap.maxiter
    if ap.kind == "laplace":
        a.tol = ap.tol
    else:  # fit_ep.method_full / method_fitc (R/gp_fit.R:150-161, R/ep.R:333-335)
        a.tol = 1e-4 if gp.method.kind == "full" else 1e-3
        a.damping = ap.damping
        a.damping_min = 0.1
        a.quad_order = ap.quad_order
    return a


def _as_x(x):
    x = np.asarray(x, dtype=np.float64)
    return x.reshape(-1, 1) if x.ndim == 1 else x


def learn_scales(gp, x):
    """learn_scales.gp (R/cf.R:831-855)."""
    for c in gp.cfs:
        c.learn_scales(x)


# ----------------------------------------------------------------------------
# fit / energy
# ----------------------------------------------------------------------------

def kmeans(x, k, init, max_iter=10, device=0):
    """Lloyd's k-means on the device (gpgp_kmeans) from the given initial centres:
    (centres k x d, iterations used, within-cluster sum of squares)."""
    x = L.fortran(_as_x(x))
    n, d = x.shape
    init = L.fortran(np.asarray(init, dtype=np.float64).reshape(k, d))
    ctx = L.default_context(device)
    centers = np.empty((k, d), order="F")
    it = C.c_int32(0)
    wss = C.c_double(0.0)
    L.check(L.load().gpgp_kmeans(ctx.h, L.ptr(x), n, d, int(k), L.ptr(init), int(max_iter),
                                 centers.ctypes.data_as(C.c_void_p), C.byref(it), C.byref(wss)), ctx.h)
    return centers, it.value, wss.value


def _kmeans_scaled(x, k, rng, device):
    """scale(x), k-means of the scaled rows (initial centres: k distinct rows drawn by
    rng, as stats::kmeans samples them), centres mapped back (R/gp_fit.R:228-233)."""
    mu = x.mean(0)
    sd = x.std(0, ddof=1) if x.shape[0] > 1 else np.ones(x.shape[1])
    xs = (x - mu) / sd
    init = xs[rng.choice(xs.shape[0], k, replace=False)]
    centers, _, _ = kmeans(xs, k, init, max_iter=10, device=device)
    return centers * sd + mu


def _bin(x, nbins, var):
    """bin (R/gp_fit.R:239-259): rows of x split into nbins equal-width bins of column var."""
    lo = x[:, var].min() - 2 * np.finfo(float).eps
    hi = x[:, var].max() + 2 * np.finfo(float).eps
    cut = np.linspace(lo, hi, nbins + 1)
    return [x[(x[:, var] > cut[i]) & (x[:, var] < cut[i + 1])] for i in range(nbins)]


def get_inducing(gp, x, device=0):
    """get_inducing (R/gp_fit.R:192-236): the given inducing inputs, or k-means centres of
    the standardised inputs (per bin of `bin_along` when set). The reference seeds R's
    stream with method$seed; numpy's generator is seeded with it here."""
    me = gp.method
    if me.inducing is not None:
        return me.inducing
    x = _as_x(x)
    rng = np.random.default_rng(me.seed)
    if me.bin_along is None:
        return _kmeans_scaled(x, me.num_inducing, rng, device)
    bins = _bin(x, me.bin_count, int(me.bin_along))
    sizes = np.array([len(b) for b in bins])
    order = np.argsort(-sizes, kind="stable")
    per_bin = np.full(me.bin_count, me.num_inducing // me.bin_count)
    per_bin[: me.num_inducing - per_bin.sum()] += 1
    zs = [_kmeans_scaled(bins[o], int(per_bin[i]), rng, device) for i, o in enumerate(order) if per_bin[i] > 0]
    return np.vstack(zs)


def gp_fit(gp, x, y, trials=None, offset=None, jitter=None, precision="fp64", device=0, grad=False):
    """gp_fit (R/gp_fit.R:54-60): posterior approximation with the current hyperparameters.

    grad=True (lik_gaussian, method_full; new, the reference has no gradient) also
    computes the energy gradient in the same call (gpgp_fit_grad): the covariance
    pass then writes K's derivative matrices beside K, and gp_energy_grad returns
    the gradient without evaluating the kernel again."""
    x = _as_x(x)
    y = np.ascontiguousarray(y, dtype=np.float64).ravel()
    n, d = x.shape
    if len(y) != n:
        raise ValueError("x and y have different numbers of rows")
    if gp.lik.kind in ("binomial", "betabinom") and trials is None:
        raise ValueError("trials must be provided for the %s likelihood." %
                         ("binomial" if gp.lik.kind == "binomial" else "beta binomial"))
    if grad and (gp.lik.kind != "gaussian" or gp.method.kind != "full"):
        raise ValueError("the energy gradient needs lik_gaussian and method_full")
    learn_scales(gp, x)
    lib = L.load()
    ctx = L.default_context(device)
    k = kernel_struct(gp.cfs, d)
    lk = _lik_struct(gp.lik)
    me, keep = _method_struct(gp, d, x)
    if gp.method.kind in RF_METHODS:
        gp.method.num_basis = check_num_basis(gp.cfs, gp.method.num_basis, d)  # R/gp_fit.R:128
        if gp.approx.kind == "ep":
            raise ValueError("approx_ep is not available for method_%s" % gp.method.kind)
    ind = None
    if gp.method.kind == "fitc":
        if gp.method.inducing is None:
            gp.method.inducing = get_inducing(gp, x, device=device)
        ind = L.fortran(gp.method.inducing)
        me.num_inducing = ind.shape[0]
        me.inducing = ind.ctypes.data
    ap = _approx_struct(gp)
    op = L.FitOpts()
    op.jitter = JITTER_DEFAULT if jitter is None else float(jitter)
    op.precision = L.PRECISION[precision]
    op.refine_iters = 2
    xf = L.fortran(x)
    tr = None if trials is None else np.ascontiguousarray(trials, dtype=np.float64)
    of = None if offset is None else np.ascontiguousarray(np.broadcast_to(offset, (n,)), dtype=np.float64)
    h = C.c_void_p()
    res = L.FitResult()
    gp._free()
    graw = None
    if grad:
        gt = np.zeros(len(_flat_terms(gp)) * L.TERM_NPARAM)
        gs = C.c_double(0.0)
        st = lib.gpgp_fit_grad(ctx.h, C.byref(k), C.byref(lk), C.byref(me), C.byref(ap), C.byref(op), L.ptr(xf),
                               n, d, L.ptr(y), L.ptr(tr), L.ptr(of), C.byref(h), C.byref(res), L.ptr(gt),
                               C.byref(gs))
        graw = (gt, gs.value)
    else:
        st = lib.gpgp_fit(ctx.h, C.byref(k), C.byref(lk), C.byref(me), C.byref(ap), C.byref(op), L.ptr(xf), n,
                          d, L.ptr(y), L.ptr(tr), L.ptr(of), C.byref(h), C.byref(res))
    L.check(st, ctx.h)
    if res.status == L.EMAXITER and gp.approx.kind == "ep":
        warnings.warn("Maximum number of iterations in EP reached")
    elif res.converged == 0 and gp.approx.kind == "laplace":
        warnings.warn("Maximum number of iterations in Laplace reached")
    gp._model = h
    gp.x = x
    gp.fit = dict(type="analytic", log_evidence=res.log_evidence, iters=res.iters,
                  quad_ok=bool(res.quad_ok), status=res.status, jitter=op.jitter, n=n,
                  converged=bool(res.converged), precision_used="mixed" if res.precision_used == 1 else "fp64",
                  y=y, trials=tr, offset=of, grad_raw=graw)
    gp.fitted = True
    return gp


def _is_fitted(gp):
    """is_fitted.gp (R/gp.R:191-205)."""
    found = isinstance(gp.fit, dict) and gp.fit.get("type") == "analytic"
    if found and not gp.fitted:
        raise RuntimeError("The GP object seems to contain a posterior fit, but is not refitted after "
                           "setting new hyperparameter values. Please refit using gp_fit after calling "
                           "set_param.")
    return found


def gp_energy(gp, include_prior=True):
    """gp_energy (R/gp.R:138-147): -log evidence - log prior."""
    if not _is_fitted(gp):
        raise RuntimeError("The GP must be fitted. Call gp_fit first.")
    e = -gp.fit["log_evidence"]
    if include_prior:
        e = e - lpdf_prior(gp)
    return e


def model_field(gp, name):
    """Copy a resident vector of the fit (alpha, fmean, z, V, fvar, cavity_mean, cavity_var;
    wmean and wcov of a method_rf / method_rbf fit)."""
    if not _is_fitted(gp):
        raise RuntimeError("The GP must be fitted. Call gp_fit first.")
    if name in ("wmean", "wcov"):
        D = int(sum(gp.method.num_basis)) if gp.method.kind in RF_METHODS else 0
        out = np.empty(D if name == "wmean" else (D, D), order="F")
        st = L.load().gpgp_model_get(gp._model, L.FIELD[name], out.ctypes.data_as(C.c_void_p))
        L.check(st, None)
        return out
    out = np.empty(gp.fit["n"])
    st = L.load().gpgp_model_get(gp._model, L.FIELD[name], L.ptr(out))
    L.check(st, None)
    return out


def gp_energy_grad(gp, include_prior=True):
    """Gradient of gp_energy with respect to the log-parameters (get_param order).

    New functionality: the reference optimises without gradients. It is
    -(1/2) tr((alpha alpha^T - C^-1) dC/dtheta) - dlog prior/dtheta, computed on
    the device for lik_gaussian with method_full.
    """
    if not _is_fitted(gp):
        raise RuntimeError("The GP must be fitted. Call gp_fit first.")
    terms = _flat_terms(gp)
    if gp.fit.get("grad_raw") is not None:  # computed with the fit (gp_fit(..., grad=True))
        gt, gsv = gp.fit["grad_raw"]
    else:
        gt = np.zeros(len(terms) * L.TERM_NPARAM)
        gs = C.c_double(0.0)
        st = L.load().gpgp_model_grad(gp._model, L.ptr(gt), C.byref(gs))
        L.check(st, None)
        gsv = gs.value
    g = []
    for ti, (grp, c) in enumerate(terms):
        if c.kind == "periodic":
            if not c.is_fixed("period"):
                g.append(gt[ti * L.TERM_NPARAM + GRAD_SLOT["period"]])
            for nme in c.base.param_names():
                g.append(gt[ti * L.TERM_NPARAM + GRAD_SLOT[nme]])
        else:
            for nme in c.param_names():
                g.append(gt[ti * L.TERM_NPARAM + GRAD_SLOT[nme]])
    if gp.lik.kind == "gaussian" and not gp.lik.is_fixed("sigma"):
        g.append(gsv)
    g = -np.array(g, dtype=np.float64)
    if include_prior:
        g = g - _dlpdf_prior(gp)
    return g


# ----------------------------------------------------------------------------
# prediction (R/gp_pred.R:88-156)
# ----------------------------------------------------------------------------

def _rf_selected(gp, cfind, d):
    """Features of the selected covariance functions (get_weight_inds, R/gp.R:235-245)."""
    nb = check_num_basis(gp.cfs, gp.method.num_basis, d)
    sel = range(len(gp.cfs)) if cfind is None else [int(k) for k in np.atleast_1d(cfind)]
    return int(sum(nb[k] for k in sel))


def _rf_prior(gp, xnew, cfind, var=False, z=None):
    """Prior variance and / or prior draws zt z of a method_rf / method_rbf model without
    a fit (gp_pred_prior / gp_draw_prior.method_rf, R/gp_pred.R:186-200, R/gp_draw.R:87-103),
    on the device. method_rbf needs the training inputs, which an unfitted model lacks."""
    if gp.method.kind == "rbf" and gp.x is None:
        raise RuntimeError("Cannot compute RBF feature map when the x matrix is not known.")
    m, d = xnew.shape
    k = kernel_struct(gp.cfs, d)
    me, keep = _method_struct(gp, d, gp.x)
    ctx = L.default_context()
    v = np.empty(m) if var else None
    draws = 0 if z is None else z.shape[1]
    sample = None if z is None else np.empty((m, draws), order="F")
    xf = L.fortran(xnew)
    st = L.load().gpgp_rf_prior(ctx.h, C.byref(k), C.byref(me), L.ptr(xf), m, d, _group_mask(gp, cfind),
                                L.ptr(v), None if z is None else z.ctypes.data_as(C.c_void_p), draws,
                                None if sample is None else sample.ctypes.data_as(C.c_void_p))
    L.check(st, ctx.h)
    del keep
    return v, sample


def _group_mask(gp, cfind):
    if cfind is None:
        return 0
    m = 0
    for k in np.atleast_1d(cfind):
        m |= 1 << int(k)
    return m


def _eval_cf(cfs, x1, x2, diag_only=False, cfind_mask=0, device=0):
    x1 = _as_x(x1)
    x2 = _as_x(x2)
    d = x1.shape[1]
    k = kernel_struct(cfs, d)
    n1, n2 = x1.shape[0], x2.shape[0]
    out = np.empty(min(n1, n2)) if diag_only else np.empty((n1, n2), order="F")
    ctx = L.default_context(device)
    a, b = L.fortran(x1), L.fortran(x2)
    st = L.load().gpgp_eval_cf(ctx.h, C.byref(k), L.ptr(a), n1, L.ptr(b), n2, d, int(diag_only),
                               cfind_mask, out.ctypes.data_as(C.c_void_p))
    L.check(st, ctx.h)
    return out


def eval_cf(cfs, x1, x2, cfind=None, diag_only=False):
    """eval_cf.list (R/cf.R:402-411) on the device; cfs is a covariance function or a list."""
    if isinstance(cfs, Cf):
        cfs = [cfs]
    mask = 0 if cfind is None else sum(1 << int(k) for k in np.atleast_1d(cfind))
    return _eval_cf(list(cfs), x1, x2, diag_only, mask)


def gp_pred(gp, xnew, var=False, quantiles=None, transform=False, cfind=None, jitter=None,
            quad_order=15, offset=None):
    """gp_pred (R/gp_pred.R:88-122)."""
    from scipy.stats import norm

    xnew = _as_x(xnew)
    if quantiles is not None or transform:
        var = True
    m = xnew.shape[0]
    if not _is_fitted(gp):
        # gp_pred_prior.method_full / method_fitc (R/gp_pred.R:142-184)
        pred = dict(mean=np.zeros(m))
        if var and gp.method.kind in RF_METHODS:
            # gp_pred_prior.method_rf (R/gp_pred.R:186-200): diag(zt zt^T)
            pred["var"] = _rf_prior(gp, xnew, cfind, var=True)[0]
        elif var:
            if gp.method.kind == "fitc" and gp.method.inducing is None:
                raise RuntimeError("Inducing points not set yet.")
            if gp.method.kind == "fitc":
                raise NotImplementedError("prior prediction with method_fitc")
            pred["var"] = eval_cf(gp.cfs, xnew, xnew, cfind, diag_only=True)
    else:
        mean = np.empty(m)
        vv = np.empty(m) if var else None
        xf = L.fortran(xnew)
        st = L.load().gpgp_pred(gp._model, L.ptr(xf), m, _group_mask(gp, cfind), L.ptr(mean), L.ptr(vv))
        L.check(st, None)
        pred = dict(mean=mean)
        if var:
            pred["var"] = vv
    if offset is not None:
        pred["mean"] = pred["mean"] + offset
    if quantiles is not None:
        q = np.stack([norm.ppf(qq, loc=pred["mean"], scale=np.sqrt(pred["var"])) for qq in quantiles], 1)
        if transform:
            q = gp.lik.response(q)
        pred["quantiles"] = q
    if transform:
        x, w = gauss_hermite_points(quad_order)
        fg = x[None, :] * np.sqrt(pred["var"])[:, None] + pred["mean"][:, None]
        ft = gp.lik.response(fg)
        mt = ft @ w
        pred["mean"] = mt
        pred["var"] = ((ft - mt[:, None]) ** 2) @ w
    return pred


def gauss_hermite_points(p):
    """gauss_hermite_points (R/quadrature.R:28-34) on the host (used by transform)."""
    c = np.zeros((p + 1, p + 1))
    c[0, 0] = 1.0
    if p >= 1:
        c[1, 1] = 1.0
    for i in range(2, p + 1):
        c[i, 1:] = c[i - 1, :-1]
        c[i, :] -= (i - 1) * c[i - 2, :]
    x = np.sort(np.real(np.roots(c[p, ::-1])))
    for _ in range(3):
        x = x - np.polyval(c[p, ::-1], x) / np.polyval(np.polyder(c[p, ::-1]), x)
    w = math.factorial(p) / (p * p * np.polyval(c[p - 1, ::-1], x) ** 2)
    return x, w


# ----------------------------------------------------------------------------
# LOO (R/gp_loo.R:73-175)
# ----------------------------------------------------------------------------

def _response(lik, f):
    """get_response (R/lik.R:460-498): the inverse link applied to latent values."""
    if lik.link == "identity":
        return f
    if lik.link == "logit":
        return 1.0 / (1.0 + np.exp(-f))
    if lik.link == "probit":
        from scipy.stats import norm
        return norm.cdf(f)
    return np.exp(f)


def _generate_target(lik, f, rng, trials=None):
    """generate_target (R/lik.R:504-537): observations drawn given latent values."""
    if lik.kind == "gaussian":
        return rng.standard_normal(f.shape) * lik.sigma + f
    mu = _response(lik, f)
    if lik.kind == "bernoulli":
        return rng.binomial(1, mu).astype(float)
    if lik.kind == "binomial":
        t = np.broadcast_to(np.asarray(trials, dtype=np.int64).reshape(-1, 1), f.shape)
        return rng.binomial(t, mu).astype(float)
    if lik.kind == "poisson":
        return rng.poisson(mu).astype(float)
    a, b = mu / lik.phi, (1 - mu) / lik.phi
    t = np.broadcast_to(np.asarray(trials, dtype=np.int64).reshape(-1, 1), f.shape)
    return rng.binomial(t, rng.beta(a, b)).astype(float)


def gp_pred_cov(gp, xnew, cfind=None, jitter=None):
    """gp_pred_post(cov = TRUE) / gp_pred_prior(cov = TRUE) (R/gp_pred.R:140-184,
    202-276): mean and the full covariance + jitter I, for method_full and
    method_fitc."""
    xnew = _as_x(xnew)
    m = xnew.shape[0]
    jit = JITTER_DEFAULT if jitter is None else float(jitter)
    if not _is_fitted(gp):
        if gp.method.kind == "fitc":  # gp_pred_prior.method_fitc (R/gp_pred.R:158-184)
            if gp.method.inducing is None:
                raise RuntimeError("Inducing points not set yet.")
            z = _as_x(gp.method.inducing)
            Kz = eval_cf(gp.cfs, z, z) + jit * np.eye(z.shape[0])
            Ktz = eval_cf(gp.cfs, xnew, z)
            Lz = np.linalg.cholesky(Kz)
            from scipy.linalg import solve_triangular
            aux = solve_triangular(Lz, Ktz.T, lower=True)
            D = eval_cf(gp.cfs, xnew, xnew, diag_only=True) - (aux * aux).sum(0)
            return np.zeros(m), aux.T @ aux + np.diag(D) + jit * np.eye(m)
        return np.zeros(m), eval_cf(gp.cfs, xnew, xnew, cfind) + jit * np.eye(m)
    mean = np.empty(m)
    cov = np.empty((m, m), order="F")
    xf = L.fortran(xnew)
    st = L.load().gpgp_pred_cov(gp._model, L.ptr(xf), m, _group_mask(gp, cfind), jit, L.ptr(mean),
                                cov.ctypes.data_as(C.c_void_p))
    L.check(st, None)
    return mean, cov


def gp_draw(gp, xnew, draws=None, transform=True, target=False, marginal=False, cfind=None, jitter=None,
            seed=None, offset=None, trials=None, device=0):
    """gp_draw (R/gp_draw.R:1-143): draws of the latent function at xnew from the posterior
    (fitted gp) or the prior, as an m x draws matrix; transform applies the inverse link,
    target draws observations. The multivariate normal draw (Cholesky of the predictive
    covariance, mean + L z) runs on the device; R's random stream cannot be reproduced, so
    the standard normals come from numpy's generator seeded by `seed`."""
    xnew = _as_x(xnew)
    m = xnew.shape[0]
    draws = 1 if draws is None else int(draws)
    rng = np.random.default_rng(seed)
    if gp.method.kind in RF_METHODS:
        # weight space (gp_draw_prior / gp_draw_analytic.method_rf, R/gp_draw.R:87-169):
        # w = wmean + t(chol(wcov)) z (prior: w = z), sample = zt w
        ks = _rf_selected(gp, cfind, xnew.shape[1])
        z = np.asfortranarray(rng.standard_normal((ks, draws)))
        if _is_fitted(gp):
            sample = np.empty((m, draws), order="F")
            st = L.load().gpgp_rf_draw(gp._model, L.ptr(L.fortran(xnew)), m, _group_mask(gp, cfind),
                                       z.ctypes.data_as(C.c_void_p), draws, sample.ctypes.data_as(C.c_void_p))
            L.check(st, None)
        else:
            sample = _rf_prior(gp, xnew, cfind, z=z)[1]
        return _draw_out(gp, sample, offset, target, transform, rng, trials)
    z = np.asfortranarray(rng.standard_normal((m, draws)))
    if marginal and _is_fitted(gp):
        pred = gp_pred(gp, xnew, var=True, cfind=cfind)
        sample = pred["mean"][:, None] + np.sqrt(pred["var"])[:, None] * z
    else:
        mean, cov = gp_pred_cov(gp, xnew, cfind=cfind, jitter=jitter)
        ctx = L.default_context(device)
        sample = np.empty((m, draws), order="F")
        st = L.load().gpgp_mvn_draw(ctx.h, L.ptr(np.ascontiguousarray(mean)), cov.ctypes.data_as(C.c_void_p), m,
                                    z.ctypes.data_as(C.c_void_p), draws, sample.ctypes.data_as(C.c_void_p))
        L.check(st, ctx.h)
    return _draw_out(gp, sample, offset, target, transform, rng, trials)


def _draw_out(gp, sample, offset, target, transform, rng, trials):
    """add_offset, then generate_target or get_response (R/gp_draw.R:66-71)."""
    if offset is not None:
        sample = sample + np.asarray(offset, dtype=np.float64).reshape(-1, 1)
    if target:
        return _generate_target(gp.lik, sample, rng, trials)
    if transform:
        return _response(gp.lik, sample)
    return sample


def gp_loo(gp, x, y, quadrature=True, quad_order=11, draws=4000, jitter=None, seed=None, **kw):
    """gp_loo (R/gp_loo.R:73-109) on the fitted data: Gauss-Hermite quadrature of order
    quad_order, or (quadrature = False) Monte Carlo with `draws` samples of each LOO
    posterior. R draws those normals from its own stream (set.seed(seed)), which cannot
    be reproduced here; numpy's generator seeded by `seed` draws them instead, in R's
    order (an n x draws matrix filled column by column)."""
    if not _is_fitted(gp):
        raise RuntimeError("The provied GP model is not fitted. Please call gp_fit (or gp_optim) first.")
    x = _as_x(x)
    y = np.asarray(y, dtype=np.float64).ravel()
    if x.shape != gp.x.shape or not np.array_equal(x, gp.x) or not np.array_equal(y, gp.fit["y"]):
        raise ValueError("gp_loo on the device uses the data the model was fitted to")
    n = len(y)
    loos = np.empty(n)
    s = C.c_double(0.0)
    if quadrature:
        st = L.load().gpgp_loo(gp._model, int(quad_order), L.ptr(loos), C.byref(s))
    else:
        draws = int(draws)
        z = np.asfortranarray(np.random.default_rng(seed).standard_normal((n, draws)))
        st = L.load().gpgp_loo_mc(gp._model, draws, z.ctypes.data_as(C.c_void_p), L.ptr(loos), C.byref(s))
    L.check(st, None)
    return dict(loo=float(loos.sum()), sd=float(n * (np.std(loos, ddof=1) / math.sqrt(n))), loos=loos)


def gp_compare(*loos, ref=None):
    """gp_compare (R/gp_loo.R:149-175): LOO differences and their standard errors."""
    vals = np.array([r["loo"] for r in loos])
    if ref is None:
        ref = int(np.argmax(vals))
    n = len(loos[0]["loos"])
    res = np.zeros((len(loos), 2))
    for i, r in enumerate(loos):
        dd = r["loos"] - loos[ref]["loos"]
        res[i, 0] = n * dd.mean()
        res[i, 1] = n * (np.std(dd, ddof=1) / math.sqrt(n))
    return res


# ----------------------------------------------------------------------------
# optimisation (R/gp_optim.R:63-160)
# ----------------------------------------------------------------------------

def _nelder_mead(fn, x0, reltol, maxit, fnscale):
    """Nelder-Mead in the form of R's optim defaults (reflection 1, contraction 0.5,
    expansion 2, initial step 10% of the largest |x0| component or 0.1,
    convergence when the simplex spread is below reltol * (|f_low| + reltol) on
    the fnscale-scaled objective)."""
    n = len(x0)
    f = lambda p: fn(p) / fnscale  # noqa: E731
    step = 0.1 * max(np.max(np.abs(x0)), 1.0) if n else 0.1
    P = [np.array(x0, dtype=np.float64)]
    for i in range(n):
        p = P[0].copy()
        p[i] += step
        P.append(p)
    F = [f(p) for p in P]
    evals = n + 1
    conv = 1
    while evals < maxit:
        order = np.argsort(F)
        P = [P[i] for i in order]
        F = [F[i] for i in order]
        if F[-1] <= F[0] + reltol * (abs(F[0]) + reltol):
            conv = 0
            break
        cen = np.mean(P[:-1], axis=0)
        xr = cen + (cen - P[-1])
        fr = f(xr)
        evals += 1
        if fr < F[0]:
            xe = cen + 2.0 * (cen - P[-1])
            fe = f(xe)
            evals += 1
            if fe < fr:
                P[-1], F[-1] = xe, fe
            else:
                P[-1], F[-1] = xr, fr
        elif fr < F[-2]:
            P[-1], F[-1] = xr, fr
        else:
            if fr < F[-1]:
                P[-1], F[-1] = xr, fr
            xc = cen + 0.5 * (P[-1] - cen)
            fc = f(xc)
            evals += 1
            if fc < F[-1]:
                P[-1], F[-1] = xc, fc
            else:
                for i in range(1, n + 1):
                    P[i] = P[0] + 0.5 * (P[i] - P[0])
                    F[i] = f(P[i])
                    evals += 1
    i = int(np.argmin(F))
    return P[i], F[i] * fnscale, conv


def _check_convergence(lossfun, loss_opt, param_opt, delta=1e-1, tol=1e-2):
    """check_convergence (R/gp_optim.R:127-160): +-delta probes per parameter."""
    for k in range(len(param_opt)):
        dp = np.zeros(len(param_opt))
        dp[k] = delta
        if loss_opt - min(lossfun(param_opt + dp), lossfun(param_opt - dp)) > tol:
            return False, ("Not all hyperparameters have reached convergence within tolerance "
                           "tol_param = %f. Try increasing the number of restarts, or reducing tol." % delta)
    return True, "Optimization converged."


def gp_optim(gp, x, y, tol=1e-4, tol_param=1e-1, maxiter=500, restarts=1, verbose=True, warnings_=True,
             method="nelder-mead", **fit_args):
    """gp_optim (R/gp_optim.R:63-125). method="nelder-mead" follows the reference;
    method="lbfgs" uses the device energy gradient (lik_gaussian, method_full)."""
    it = [0]

    def energy(param, grad=False):
        set_param(gp, param)
        try:
            gp_fit(gp, x, y, grad=grad, **fit_args)
        except np.linalg.LinAlgError:
            return np.inf
        e = gp_energy(gp)
        if verbose:
            print(" ".join("%8.2f" % p for p in param), "%10.2f" % e, "%9d" % it[0])
        it[0] += 1
        return e

    _, p0 = get_param(gp)
    n = len(np.atleast_1d(y))
    if method == "lbfgs":
        from scipy.optimize import minimize

        def fg(param):
            # fit and gradient in one call (gpgp_fit_grad)
            e = energy(param, grad=True)
            return e, (gp_energy_grad(gp) if np.isfinite(e) else np.zeros(len(param)))

        r = minimize(fg, p0, jac=True, method="L-BFGS-B", options=dict(maxiter=maxiter, ftol=tol / n))
        p_opt, e_opt = r.x, r.fun
    else:
        p_opt, e_opt, conv = _nelder_mead(energy, p0, tol, maxiter, n)
        if conv == 1 and warnings_:
            warnings.warn("Maximum number of iterations reached, optimization may not have converged.")
    set_param(gp, p_opt)
    gp_fit(gp, x, y, **fit_args)
    if warnings_:
        ok, msg = _check_convergence(energy, e_opt, p_opt, delta=tol_param)
        set_param(gp, p_opt)
        gp_fit(gp, x, y, **fit_args)
        if not ok:
            if restarts > 0:
                return gp_optim(gp, x, y, tol=tol, tol_param=tol_param, maxiter=maxiter,
                                restarts=restarts - 1, verbose=verbose, warnings_=warnings_,
                                method=method, **fit_args)
            warnings.warn(msg)
    return gp
