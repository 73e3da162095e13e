"""Batched small GPs on the device (gpgp_batch_* of include/gpgp.h).

Each problem is the reference's gp_fit (lik_gaussian, method_full, one
covariance function over all inputs), gp_loo (approx_laplace, Gauss-Hermite
quadrature) and gp_pred with var = TRUE; all problems run as one CUDA graph.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L

KINDS = {"sexp": 2, "matern32": 3, "matern52": 4}


class BatchPlan:
    """A captured batch: construct once, then run() / upload() / results()."""

    def __init__(self, problems, precision="mixed", quad_order=11, jitter=1e-6, device=0):
        self.lib = L.load()
        self.ctx = L.default_context(device)
        self.n = len(problems)
        self._structs, self._keep = self._pack(problems)
        self.shapes = [(int(s.n), int(s.m)) for s in self._structs]
        h = C.c_void_p()
        st = self.lib.gpgp_batch_create(self.ctx.h, C.cast(self._structs, C.c_void_p), self.n,
                                        L.PRECISION[precision], int(quad_order), float(jitter), C.byref(h))
        L.check(st, self.ctx.h)
        self.h = h

    @staticmethod
    def _pack(problems):
        arr = (L.BatchProblem * len(problems))()
        keep = []
        for i, p in enumerate(problems):
            x = np.asfortranarray(np.asarray(p["x"], dtype=np.float64).reshape(len(p["y"]), -1))
            y = np.ascontiguousarray(p["y"], dtype=np.float64)
            xt = np.asfortranarray(np.asarray(p["xt"], dtype=np.float64).reshape(-1, x.shape[1]))
            keep += [x, y, xt]
            s = arr[i]
            s.n, s.d, s.m = x.shape[0], x.shape[1], xt.shape[0]
            s.kind = KINDS[p.get("kind", "sexp")]
            s.lscale, s.magn, s.sigma = float(p["lscale"]), float(p.get("magn", 1.0)), float(p["sigma"])
            s.x, s.y, s.xt = x.ctypes.data, y.ctypes.data, xt.ctypes.data
        return arr, keep

    def upload(self, problems):
        self._structs, self._keep = self._pack(problems)
        L.check(self.lib.gpgp_batch_upload(self.h, C.cast(self._structs, C.c_void_p)), self.ctx.h)

    def run(self):
        L.check(self.lib.gpgp_batch_run(self.h), self.ctx.h)

    def results(self):
        nm = sum(m for _, m in self.shapes)
        nn = sum(n for n, _ in self.shapes)
        lml, mean, var, loos = np.empty(self.n), np.empty(nm), np.empty(nm), np.empty(nn)
        L.check(self.lib.gpgp_batch_results(self.h, L.ptr(lml), L.ptr(mean), L.ptr(var), L.ptr(loos)),
                self.ctx.h)
        out, om, on = [], 0, 0
        for i, (n, m) in enumerate(self.shapes):
            out.append(dict(log_evidence=lml[i], mean=mean[om:om + m], var=var[om:om + m],
                            loos=loos[on:on + n], loo=float(loos[on:on + n].sum())))
            om += m
            on += n
        return out

    def info(self):
        nb = C.c_int32()
        self.lib.gpgp_batch_info(self.h, C.byref(nb), None, None, None, None)
        k = nb.value
        bn, bc, bv = (C.c_int32 * k)(), (C.c_int32 * k)(), (C.c_int32 * k)()
        tms = (C.c_double * 3)()
        self.lib.gpgp_batch_info(self.h, C.byref(nb), bn, bc, bv, tms)
        names = {0: "fp64-pipe", 1: "tensor-64", 2: "tensor-256"}
        return dict(buckets=[(bn[i], bc[i], names[bv[i]]) for i in range(k)], autotune_ms=list(tms))

    def close(self):
        if getattr(self, "h", None):
            self.lib.gpgp_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def gp_fit_batched(problems, precision="mixed", quad_order=11, jitter=1e-6):
    """Fit, LOO and predict every problem; returns one dict per problem."""
    plan = BatchPlan(problems, precision, quad_order, jitter)
    plan.run()
    res = plan.results()
    plan.close()
    return res
