"""Generate the golden fixtures of tests/golden from the oracle.

The reference (R gplite 0.13.0) cannot run in this environment and ships no
vectors, so the fixtures freeze the oracle's outputs on seeded synthetic inputs
that follow the workloads' stated shapes: a regression pin for the oracle and
the checked values for the CUDA library. Besides the small cases, four fixtures
are at the workloads' full sizes:
  c2_n16384    full GP regression, n = 16384, d = 8, matern52 + const: evidence,
               alpha, energy gradient, prediction at 8192 points;
  c3_n8192     Bernoulli, n = 8192, d = 4, sexp: Laplace (tol 1e-6) and EP
               (damping 0.9) iterations, evidences, latent means, LOO;
  fitc_n65536  FITC regression, n = 65536, 256 inducing inputs chosen at random,
               d = 2: evidence, latent means (every 64th), prediction at 256 points;
  c4_sample    32 small problems, two in every 64-wide size bucket from 64 to 1024:
               evidence, LOO and prediction at 128 points each.
Each full-size fixture also records the oracle's own sensitivity: the largest
relative change of each output when every input is moved by one ulp (random
sign). A test tolerance below that would test rounding, not the algorithm.
Inputs drawn from uniforms are rebuilt bit for bit by tests/golden/synth.py;
the rest (normal inputs, GP draws) are stored, rounded to float32.
Run from the repository root (about ten minutes on eight cores):
    python tests/golden/make_golden.py [c1 c3 gh c2 c3big fitc c4]
"""
import copy
import os
import sys
import time
import warnings

import numpy as np
from scipy import linalg as sla

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, HERE)
from oracle import gplite_ref as R  # noqa: E402
import synth as S  # noqa: E402

THREADS = os.cpu_count() or 1


def ulp_nudge(a, seed):
    """Every entry moved by one ulp, up or down at random."""
    rng = np.random.default_rng(seed)
    a = np.asarray(a, dtype=np.float64)
    return np.where(rng.uniform(size=a.shape) < 0.5, np.nextafter(a, np.inf), np.nextafter(a, -np.inf))


def relmax(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def relmax_finite(a, b):
    """relmax over the entries where both are finite (the reference's LOO variance
    1 / (1 / post_var - 1 / V) can cancel to a negative value for tiny sigma, and the
    density is NaN there)."""
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    ok = np.isfinite(a) & np.isfinite(b)
    return relmax(a[ok], b[ok]) if ok.any() else 0.0


def rel_elem(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300)))


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


def gp_draw_f32(cfs, x, seed, noise=0.0):
    """A draw of the GP (FP64 Cholesky of K + 1e-6 I) plus N(0, noise^2), rounded to float32."""
    rng = np.random.default_rng(seed)
    K = R.eval_cf(cfs, x, x, threads=THREADS)
    K[np.diag_indices(len(x))] += 1e-6
    f = sla.cholesky(K, lower=True, overwrite_a=True, check_finite=False) @ rng.standard_normal(len(x))
    return S.to_f32_exact(f + noise * rng.standard_normal(len(x)))


# ---------------------------------------------------------------------------
# full-size fixtures
# ---------------------------------------------------------------------------

def c2_cfs():
    return [R.cf("matern52", lscale=S.C2_LSCALE, magn=S.C2_MAGN), R.cf("const", magn=S.C2_CMAGN)]


def c2_run(x, y, xt):
    gp = R.gp_init(c2_cfs(), R.lik("gaussian", sigma=S.C2_SIGMA))
    gp = R.gp_fit(gp, x, y, threads=THREADS)
    g = R.gp_energy_grad(gp, threads=THREADS)
    Kt = R.eval_cf(gp.cfs, xt, x, threads=THREADS)
    mean = Kt @ gp.fit["alpha"]
    aux = sla.solve_triangular(gp.fit["C_chol"], Kt.T, lower=True, overwrite_b=True, check_finite=False)
    del Kt
    var = R.eval_cf(gp.cfs, xt, xt, diag_only=True) - (aux * aux).sum(0)
    return dict(lml=gp.fit["log_evidence"], alpha=gp.fit["alpha"], grad=g, mean=mean, var=var)


def c2():
    x, xt = S.c2_inputs()
    y = gp_draw_f32(c2_cfs(), x, 21, noise=S.C2_SIGMA)
    out = c2_run(x, y, xt)
    nud = c2_run(ulp_nudge(x, 1), ulp_nudge(y, 2), ulp_nudge(xt, 3))
    sens = dict(sens_lml=rel_elem(nud["lml"], out["lml"]), sens_alpha=relmax(nud["alpha"], out["alpha"]),
                sens_grad=rel_elem(nud["grad"], out["grad"]), sens_mean=relmax(nud["mean"], out["mean"]),
                sens_var=relmax(nud["var"], out["var"]))
    return dict(y=y.astype(np.float32), **out, **sens)


def c3_run(x, y):
    out = {}
    for pre, ap in (("la_", R.approx_laplace(tol=1e-6)), ("ep_", R.approx_ep(damping=0.9))):
        gp = R.gp_init([R.cf("sexp", lscale=0.5, magn=2.0)], R.lik("bernoulli"), approx=ap)
        gp = R.gp_fit(gp, x, y, threads=THREADS)
        out.update({pre + "lml": gp.fit["log_evidence"], pre + "fmean": gp.fit["fmean"],
                    pre + "iters": gp.fit["iters"], pre + "loos": R.gp_loo(gp, x, y)["loos"]})
    return out


def c3_big():
    """C3: n = 8192, x ~ N(0, I_4), f ~ GP(sexp(0.5, 2)), y ~ Bernoulli(logistic(f))."""
    n, d = 8192, 4
    rng = np.random.default_rng(30)
    x = S.to_f32_exact(rng.standard_normal((n, d)))
    f = gp_draw_f32([R.cf("sexp", lscale=0.5, magn=2.0)], x, 31)
    y = (rng.uniform(size=n) < 1 / (1 + np.exp(-f))).astype(np.float64)
    out = c3_run(x, y)
    nud = c3_run(ulp_nudge(x, 4), y)
    sens = {}
    for pre in ("la_", "ep_"):
        sens["sens_" + pre + "lml"] = rel_elem(nud[pre + "lml"], out[pre + "lml"])
        sens["sens_" + pre + "fmean"] = relmax(nud[pre + "fmean"], out[pre + "fmean"])
        sens["sens_" + pre + "loos"] = relmax(nud[pre + "loos"], out[pre + "loos"])
        sens["sens_" + pre + "iters"] = int(nud[pre + "iters"] != out[pre + "iters"])
    return dict(x=x.astype(np.float32), y=y.astype(np.uint8), **out, **sens)


FITC_LSCALE, FITC_SIGMA = 0.7, 0.1


def fitc_run(x, z, xt, y):
    gp = R.gp_init([R.cf("sexp", lscale=FITC_LSCALE, magn=1.0)], R.lik("gaussian", sigma=FITC_SIGMA),
                   method=R.method_fitc(z))
    gp = R.gp_fit(gp, x, y)
    p = R.gp_pred(gp, xt, var=True)
    return dict(lml=gp.fit["log_evidence"], fmean_s64=gp.fit["fmean"][::64], mean=p["mean"], var=p["var"])


def fitc():
    """C5's FITC request: n = 65536, d = 2, sexp(0.7), lik_gaussian(0.1), 256 inducing inputs
    chosen at random among x. The latent function is a draw of the FITC prior itself
    (Kxz Kz^-1/2 w + sqrt(D) v), which needs no n x n Cholesky."""
    x, z, xt = S.fitc_inputs()
    rng = np.random.default_rng(53)
    cfs = [R.cf("sexp", lscale=FITC_LSCALE, magn=1.0)]
    Kz, Kxz, Kz_chol, K_diag, D = R.fitc_prepare(cfs, x, z, 1e-6)
    f = Kxz @ sla.solve_triangular(Kz_chol.T, rng.standard_normal(len(z)), lower=False) \
        + np.sqrt(np.maximum(D, 0)) * rng.standard_normal(len(x))
    y = S.to_f32_exact(f + FITC_SIGMA * rng.standard_normal(len(x)))
    out = fitc_run(x, z, xt, y)
    nud = fitc_run(ulp_nudge(x, 5), ulp_nudge(z, 6), ulp_nudge(xt, 7), ulp_nudge(y, 8))
    sens = dict(sens_lml=rel_elem(nud["lml"], out["lml"]), sens_fmean=relmax(nud["fmean_s64"], out["fmean_s64"]),
                sens_mean=relmax(nud["mean"], out["mean"]), sens_var=relmax(nud["var"], out["var"]))
    return dict(y=y.astype(np.float32), **out, **sens)


def c4_run(p, y, x=None, xt=None):
    x = p["x"] if x is None else x
    xt = p["xt"] if xt is None else xt
    gp = R.gp_init([R.cf(p["kind"], lscale=p["lscale"], magn=1.0)], R.lik("gaussian", sigma=p["sigma"]))
    gp = R.gp_fit(gp, x, y)
    pr = R.gp_pred(gp, xt, var=True)
    return gp.fit["log_evidence"], R.gp_loo(gp, x, y)["loos"], pr["mean"], pr["var"]


def c4():
    ys, lml, loos, mean, var, sl, sloo, smean, svar = [], [], [], [], [], [], [], [], []
    for i, n in enumerate(S.C4_SIZES):
        p = S.c4_problem(i, n)
        y = gp_draw_f32([R.cf(p["kind"], lscale=p["lscale"], magn=1.0)], p["x"], 700 + i, noise=p["sigma"])
        a = c4_run(p, y)
        # the largest change over four independent one-ulp nudges: the LOO variance
        # 1 / (1 / post_var - 1 / V) cancels for small sigma, and a single nudge can
        # land on a lucky rounding
        bs = [c4_run(p, ulp_nudge(y, 800 + i + 97 * k), ulp_nudge(p["x"], 900 + i + 97 * k),
                     ulp_nudge(p["xt"], 1000 + i + 97 * k)) for k in range(4)]
        ys.append(y)
        lml.append(a[0])
        loos.append(a[1])
        mean.append(a[2])
        var.append(a[3])
        sl.append(max(abs(b[0] - a[0]) / max(abs(a[0]), n) for b in bs))
        sloo.append(max(relmax_finite(b[1], a[1]) for b in bs))
        smean.append(max(relmax(b[2], a[2]) for b in bs))
        svar.append(max(relmax(b[3], a[3]) for b in bs))
    return dict(y=np.concatenate(ys).astype(np.float32), lml=np.array(lml), loos=np.concatenate(loos),
                mean=np.concatenate(mean), var=np.concatenate(var), sens_lml=np.array(sl),
                sens_loos=np.array(sloo), sens_mean=np.array(smean), sens_var=np.array(svar))


def main():
    which = sys.argv[1:] or ["c1", "c3", "gh", "c2", "c3big", "fitc", "c4"]
    warnings.simplefilter("ignore")
    jobs = {
        "c1": ("c1_gauss_n200.npz", c1),
        "c3": ("c3_bernoulli_n256.npz", c3_small),
        "c2": ("c2_n16384.npz", c2),
        "c3big": ("c3_n8192.npz", c3_big),
        "fitc": ("fitc_n65536.npz", fitc),
        "c4": ("c4_sample.npz", c4),
    }
    for w in which:
        t0 = time.time()
        if w == "gh":
            x, wt = R.gauss_hermite_points(11)
            np.savez_compressed(os.path.join(HERE, "gh.npz"), x11=x, w11=wt,
                                x15=R.gauss_hermite_points(15)[0], w15=R.gauss_hermite_points(15)[1])
        else:
            name, fn = jobs[w]
            np.savez_compressed(os.path.join(HERE, name), **fn())
        print("%s written in %.0f s" % (w, time.time() - t0), flush=True)


if __name__ == "__main__":
    main()
