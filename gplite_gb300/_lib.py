"""ctypes binding of libgpgp.so (the C ABI declared in include/gpgp.h).

The shared library is built in-tree by ``gplite_gb300/build.py``. There is no
fallback: if the library is missing, importing the compute entry points raises.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgpgp.so")

MAX_VARS = 16
MAX_TERMS = 16
TERM_NPARAM = 5

# enums (include/gpgp.h)
OK, ENOT_PD, ENAN, EMAXITER, EUNSUPPORTED, EOOM, ETIMEOUT, ECUDA, EINVAL, ENOT_FITTED, EBUSY = range(11)
CF_KIND = {"const": 0, "lin": 1, "sexp": 2, "matern32": 3, "matern52": 4, "nn": 5}
LIK_KIND = {"gaussian": 0, "bernoulli": 1, "binomial": 2, "poisson": 3, "betabinom": 4}
LINK = {"identity": 0, "logit": 1, "probit": 2, "log": 3}
METHOD = {"full": 0, "fitc": 1, "rf": 2, "rbf": 3}
APPROX = {"laplace": 0, "ep": 1}
PRECISION = {"fp64": 0, "mixed": 1}
PHASES = ["cov", "potrf", "solve", "trtri", "lauum", "grad", "pred_mean", "pred_var"]
FIELD = {"alpha": 0, "fmean": 1, "z": 2, "V": 3, "fvar": 4, "cavity_mean": 5, "cavity_var": 6, "wmean": 7,
         "wcov": 8}


class CfTerm(C.Structure):
    _fields_ = [("kind", C.c_int32), ("group", C.c_int32), ("periodic", C.c_int32),
                ("normalize", C.c_int32), ("nvars", C.c_int32), ("vars", C.c_int32 * MAX_VARS),
                ("means", C.c_double * MAX_VARS), ("scales", C.c_double * MAX_VARS),
                ("lscale", C.c_double), ("magn", C.c_double), ("sigma0", C.c_double),
                ("sigma", C.c_double), ("period", C.c_double)]


class Kernel(C.Structure):
    _fields_ = [("nterms", C.c_int32), ("ngroups", C.c_int32), ("term", CfTerm * MAX_TERMS)]


class Lik(C.Structure):
    _fields_ = [("kind", C.c_int32), ("link", C.c_int32), ("sigma", C.c_double), ("phi", C.c_double)]


class Method(C.Structure):
    _fields_ = [("kind", C.c_int32), ("num_inducing", C.c_int32), ("inducing", C.c_void_p),
                ("num_basis", C.c_int32 * MAX_TERMS), ("draws", C.c_void_p * MAX_TERMS)]


class Approx(C.Structure):
    _fields_ = [("kind", C.c_int32), ("maxiter", C.c_int32), ("tol", C.c_double),
                ("damping", C.c_double), ("damping_min", C.c_double), ("quad_order", C.c_int32)]


class FitOpts(C.Structure):
    _fields_ = [("jitter", C.c_double), ("precision", C.c_int32), ("refine_iters", C.c_int32)]


class FitResult(C.Structure):
    _fields_ = [("log_evidence", C.c_double), ("status", C.c_int32), ("iters", C.c_int32),
                ("info", C.c_int64), ("quad_ok", C.c_int32), ("converged", C.c_int32),
                ("precision_used", C.c_int32)]


class BatchProblem(C.Structure):
    _fields_ = [("n", C.c_int32), ("d", C.c_int32), ("m", C.c_int32), ("kind", C.c_int32),
                ("lscale", C.c_double), ("magn", C.c_double), ("sigma", C.c_double),
                ("x", C.c_void_p), ("y", C.c_void_p), ("xt", C.c_void_p)]


class ServerOpts(C.Structure):
    _fields_ = [("device", C.c_int32), ("workers", C.c_int32), ("hbm_budget", C.c_int64),
                ("precision", C.c_int32), ("batch_max_n", C.c_int32), ("batch_max", C.c_int32),
                ("jitter", C.c_double)]


class Request(C.Structure):
    _fields_ = [("kernel", C.c_void_p), ("lik", C.c_void_p), ("method", C.c_void_p), ("approx", C.c_void_p),
                ("x", C.c_void_p), ("n", C.c_int64), ("d", C.c_int32), ("y", C.c_void_p),
                ("trials", C.c_void_p), ("offset", C.c_void_p), ("xt", C.c_void_p), ("m", C.c_int64),
                ("keep", C.c_int32), ("model", C.c_int64), ("mean", C.c_void_p), ("var", C.c_void_p)]


class RequestResult(C.Structure):
    _fields_ = [("status", C.c_int32), ("lane", C.c_int32), ("log_evidence", C.c_double),
                ("converged", C.c_int32), ("iters", C.c_int32), ("precision_used", C.c_int32),
                ("reserved", C.c_int32), ("model", C.c_int64), ("queue_ms", C.c_double),
                ("run_ms", C.c_double), ("total_ms", C.c_double)]


class ServerStats(C.Structure):
    _fields_ = [(k, C.c_int64) for k in ("submitted", "completed", "failed", "pending", "inflight", "batches",
                                         "batched_requests", "bytes_inflight", "bytes_resident", "bytes_peak",
                                         "budget")] + [("p50_ms", C.c_double), ("p99_ms", C.c_double),
                                                       ("max_ms", C.c_double)]


_P = C.c_void_p
_D = C.POINTER(C.c_double)

# name -> (restype, argtypes); the list of every symbol include/gpgp.h declares
SIGNATURES = {
    "gpgp_create": (C.c_int, [C.POINTER(_P), C.c_int]),
    "gpgp_destroy": (C.c_int, [_P]),
    "gpgp_status_string": (C.c_char_p, [C.c_int]),
    "gpgp_last_error": (C.c_char_p, [_P]),
    "gpgp_launch_count": (C.c_int64, [_P]),
    "gpgp_sync": (C.c_int, [_P]),
    "gpgp_stream": (_P, [_P]),
    "gpgp_profile_enable": (C.c_int, [_P, C.c_int32]),
    "gpgp_profile_read": (C.c_int, [_P, _P, _P]),
    "gpgp_kernel_profile_read": (C.c_int, [_P, C.c_int32, _P, _P, _P]),
    "gpgp_cf_sexp": (C.c_int, [_P, C.c_int64, _P, C.c_int64, C.c_int32, C.c_double, C.c_double, C.c_int32, _P]),
    "gpgp_cf_matern32": (C.c_int, [_P, C.c_int64, _P, C.c_int64, C.c_int32, C.c_double, C.c_double, C.c_int32, _P]),
    "gpgp_cf_matern52": (C.c_int, [_P, C.c_int64, _P, C.c_int64, C.c_int32, C.c_double, C.c_double, C.c_int32, _P]),
    "gpgp_cf_nn": (C.c_int, [_P, C.c_int64, _P, C.c_int64, C.c_int32, C.c_double, C.c_double, C.c_double, C.c_int32, _P]),
    "gpgp_eval_cf": (C.c_int, [_P, C.POINTER(Kernel), _P, C.c_int64, _P, C.c_int64, C.c_int32, C.c_int32, C.c_uint32, _P]),
    "gpgp_fit": (C.c_int, [_P, C.POINTER(Kernel), C.POINTER(Lik), C.POINTER(Method), C.POINTER(Approx),
                           C.POINTER(FitOpts), _P, C.c_int64, C.c_int32, _P, _P, _P, C.POINTER(_P),
                           C.POINTER(FitResult)]),
    "gpgp_fit_dev": (C.c_int, [_P, C.POINTER(Kernel), C.POINTER(Lik), C.POINTER(Method), C.POINTER(Approx),
                               C.POINTER(FitOpts), _P, C.c_int64, C.c_int32, _P, _P, _P, C.POINTER(_P),
                               C.POINTER(FitResult)]),
    "gpgp_model_free": (C.c_int, [_P]),
    "gpgp_model_grad": (C.c_int, [_P, _P, _P]),
    "gpgp_fit_grad": (C.c_int, [_P, C.POINTER(Kernel), C.POINTER(Lik), C.POINTER(Method), C.POINTER(Approx),
                                C.POINTER(FitOpts), _P, C.c_int64, C.c_int32, _P, _P, _P, C.POINTER(_P),
                                C.POINTER(FitResult), _P, _P]),
    "gpgp_fit_grad_dev": (C.c_int, [_P, C.POINTER(Kernel), C.POINTER(Lik), C.POINTER(Method), C.POINTER(Approx),
                                    C.POINTER(FitOpts), _P, C.c_int64, C.c_int32, _P, _P, _P, C.POINTER(_P),
                                    C.POINTER(FitResult), _P, _P]),
    "gpgp_model_get": (C.c_int, [_P, C.c_int32, _P]),
    "gpgp_pred": (C.c_int, [_P, _P, C.c_int64, C.c_uint32, _P, _P]),
    "gpgp_pred_dev": (C.c_int, [_P, _P, C.c_int64, C.c_uint32, _P, _P]),
    "gpgp_loo": (C.c_int, [_P, C.c_int32, _P, _P]),
    "gpgp_loo_mc": (C.c_int, [_P, C.c_int64, _P, _P, _P]),
    "gpgp_pred_cov": (C.c_int, [_P, _P, C.c_int64, C.c_uint32, C.c_double, _P, _P]),
    "gpgp_kmeans": (C.c_int, [_P, _P, C.c_int64, C.c_int32, C.c_int32, _P, C.c_int32, _P, _P, _P]),
    "gpgp_mvn_draw": (C.c_int, [_P, _P, _P, C.c_int64, _P, C.c_int64, _P]),
    "gpgp_rf_prior": (C.c_int, [_P, C.POINTER(Kernel), C.POINTER(Method), _P, C.c_int64, C.c_int32, C.c_uint32,
                                _P, _P, C.c_int64, _P]),
    "gpgp_rf_draw": (C.c_int, [_P, _P, C.c_int64, C.c_uint32, _P, C.c_int64, _P]),
    "gpgp_batch_create": (C.c_int, [_P, _P, C.c_int32, C.c_int32, C.c_int32, C.c_double, C.POINTER(_P)]),
    "gpgp_batch_upload": (C.c_int, [_P, _P]),
    "gpgp_batch_run": (C.c_int, [_P]),
    "gpgp_batch_results": (C.c_int, [_P, _P, _P, _P, _P]),
    "gpgp_batch_info": (C.c_int, [_P, _P, _P, _P, _P, _P]),
    "gpgp_batch_destroy": (C.c_int, [_P]),
    "gpgp_server_create": (C.c_int, [C.POINTER(ServerOpts), C.POINTER(_P)]),
    "gpgp_server_submit": (C.c_int, [_P, C.POINTER(Request), C.POINTER(C.c_int64)]),
    "gpgp_server_poll": (C.c_int, [_P, C.c_int64, C.c_int32, C.POINTER(RequestResult)]),
    "gpgp_server_release": (C.c_int, [_P, C.c_int64]),
    "gpgp_server_stats_get": (C.c_int, [_P, C.POINTER(ServerStats)]),
    "gpgp_server_destroy": (C.c_int, [_P]),
    "gpgp_mixed_selftest": (C.c_int, [_P, C.c_int64, C.c_int64, C.c_int64, C.c_int32, _P]),
    "gpgp_cov_df_selftest": (C.c_int, [_P, C.POINTER(Kernel), _P, C.c_int64, C.c_int32, C.c_double, _P]),
    "gpgp_wait_selftest": (C.c_int, [_P, C.c_int32]),
    "gpgp_fit_gaussian_noalloc": (C.c_int, [_P, C.POINTER(Kernel), C.c_double, C.c_double, _P, C.c_int64,
                                            C.c_int32, _P, _P, _P]),
}

_lib = None
_lock = threading.Lock()


class GpgpError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s (status %d): %s" % (STATUS_NAMES.get(status, "?"), status, msg))
        self.status = status


class NotPositiveDefinite(GpgpError, np.linalg.LinAlgError):
    pass


STATUS_NAMES = {OK: "ok", ENOT_PD: "not positive definite", ENAN: "NaN", EMAXITER: "max iterations",
                EUNSUPPORTED: "unsupported", EOOM: "out of memory", ETIMEOUT: "timeout",
                ECUDA: "CUDA error", EINVAL: "invalid argument", ENOT_FITTED: "not fitted",
                EBUSY: "busy"}


def load(path: str = LIB_PATH):
    """Load libgpgp.so and declare every signature. Raises if the library is absent."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(path):
            raise ImportError("libgpgp.so is not built (%s); run gplite_gb300/build.py or "
                              "__graft_entry__.build() first" % path)
        lib = C.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        _lib = lib
        return lib


def check(st, ctx=None):
    if st == OK:
        return
    lib = load()
    msg = lib.gpgp_last_error(ctx)
    msg = msg.decode() if msg else ""
    if st == ENOT_PD:
        raise NotPositiveDefinite(st, msg)
    raise GpgpError(st, msg)


def ptr(a):
    """Host pointer of a C-contiguous float64 array (or None)."""
    if a is None:
        return None
    return a.ctypes.data_as(C.c_void_p)


def fortran(a):
    """Column-major float64 copy of a 2-D array (R matrix layout)."""
    return np.asfortranarray(np.asarray(a, dtype=np.float64))


class Context:
    """One device, one stream (gpgp_ctx)."""

    def __init__(self, device: int = 0):
        lib = load()
        h = C.c_void_p()
        st = lib.gpgp_create(C.byref(h), device)
        check(st, None)
        self.h = h
        self.device = device

    def close(self):
        if self.h:
            load().gpgp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def sync(self):
        check(load().gpgp_sync(self.h), self.h)

    @property
    def stream(self):
        return load().gpgp_stream(self.h)


_default_ctx = {}


def default_context(device: int = 0) -> Context:
    with _lock:
        c = _default_ctx.get(device)
    if c is None:
        c = Context(device)
        with _lock:
            _default_ctx[device] = c
    return c


def launch_count() -> int:
    return int(load().gpgp_launch_count(None))
