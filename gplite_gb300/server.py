"""Request server (gpgp_server_* of include/gpgp.h): fit + predict requests of
mixed size served with continuous batching, HBM-budgeted admission and
resident models.

Each request is what one ``gp_fit`` (R/gp_fit.R:54-60) followed by
``gp_pred(var=TRUE)`` (R/gp_pred.R:88-122) computes for a gp object of
``gp_init``; a kept model answers later ``gp_pred`` requests without a refit.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from . import gp as _gp


class Ticket:
    """A submitted request: its id and the buffers the server writes into."""

    def __init__(self, rid, m, mean, var, keepalive):
        self.id = rid
        self.m = m
        self.mean = mean
        self.var = var
        self._keepalive = keepalive


class GPServer:
    def __init__(self, precision="fp64", workers=4, hbm_budget=0, batch_max_n=1024, batch_max=4096,
                 jitter=1e-6, device=0):
        self.lib = L.load()
        o = L.ServerOpts()
        o.device = device
        o.workers = workers
        o.hbm_budget = int(hbm_budget)
        o.precision = L.PRECISION[precision]
        o.batch_max_n = batch_max_n
        o.batch_max = batch_max
        o.jitter = jitter
        h = C.c_void_p()
        L.check(self.lib.gpgp_server_create(C.byref(o), C.byref(h)), None)
        self.h = h

    def submit(self, gp, x, y, xt=None, keep=False, trials=None, offset=None, want_var=True):
        """Queue gp_fit(gp, x, y) and, with xt, gp_pred(gp, xt, var=want_var)."""
        x = _gp._as_x(x)
        n, d = x.shape
        y = np.ascontiguousarray(y, dtype=np.float64).ravel()
        _gp.learn_scales(gp, x)
        k = _gp.kernel_struct(gp.cfs, d)
        lk = _gp._lik_struct(gp.lik)
        me = L.Method()
        me.kind = L.METHOD[gp.method.kind]
        ind = None
        if gp.method.kind == "fitc":
            ind = L.fortran(gp.method.inducing)
            me.num_inducing = ind.shape[0]
            me.inducing = ind.ctypes.data
        ap = _gp._approx_struct(gp)
        xf = L.fortran(x)
        xt = None if xt is None else L.fortran(_gp._as_x(xt))
        m = 0 if xt is None else xt.shape[0]
        mean = np.empty(m)
        var = np.empty(m) if want_var else None
        tr = None if trials is None else np.ascontiguousarray(trials, dtype=np.float64)
        of = None if offset is None else np.ascontiguousarray(np.broadcast_to(offset, (n,)), dtype=np.float64)
        q = L.Request()
        q.kernel, q.lik = C.addressof(k), C.addressof(lk)
        q.method, q.approx = C.addressof(me), C.addressof(ap)
        q.x, q.n, q.d, q.y = xf.ctypes.data, n, d, y.ctypes.data
        q.trials = None if tr is None else tr.ctypes.data
        q.offset = None if of is None else of.ctypes.data
        q.xt = None if xt is None else xt.ctypes.data
        q.m = m
        q.keep = 1 if keep else 0
        q.model = -1
        q.mean = mean.ctypes.data
        q.var = None if var is None else var.ctypes.data
        rid = C.c_int64(-1)
        L.check(self.lib.gpgp_server_submit(self.h, C.byref(q), C.byref(rid)), None)
        return Ticket(rid.value, m, mean, var, None)

    def submit_pred(self, model, xt, want_var=True):
        """Queue gp_pred on a model kept resident by an earlier request."""
        xt = L.fortran(_gp._as_x(xt))
        m = xt.shape[0]
        mean = np.empty(m)
        var = np.empty(m) if want_var else None
        q = L.Request()
        q.xt, q.m, q.model = xt.ctypes.data, m, int(model)
        q.mean = mean.ctypes.data
        q.var = None if var is None else var.ctypes.data
        rid = C.c_int64(-1)
        L.check(self.lib.gpgp_server_submit(self.h, C.byref(q), C.byref(rid)), None)
        return Ticket(rid.value, m, mean, var, None)

    def poll(self, ticket, wait_ms=-1):
        """The request's result once it is done (None while it is not)."""
        r = L.RequestResult()
        st = self.lib.gpgp_server_poll(self.h, ticket.id, int(wait_ms), C.byref(r))
        if st == L.EBUSY:
            return None
        L.check(st, None)
        return dict(status=r.status, lane="batch" if r.lane == 0 else "worker", log_evidence=r.log_evidence,
                    converged=bool(r.converged), iters=r.iters,
                    precision_used="mixed" if r.precision_used == 1 else "fp64",
                    model=r.model, queue_ms=r.queue_ms, run_ms=r.run_ms, total_ms=r.total_ms,
                    mean=ticket.mean, var=ticket.var)

    def release(self, model):
        L.check(self.lib.gpgp_server_release(self.h, int(model)), None)

    def stats(self):
        s = L.ServerStats()
        L.check(self.lib.gpgp_server_stats_get(self.h, C.byref(s)), None)
        return {name: getattr(s, name) for name, _ in L.ServerStats._fields_}

    def close(self):
        if self.h:
            self.lib.gpgp_server_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
