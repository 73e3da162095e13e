"""Self-test of the sliced tensor-core GEMM on the local GPU.

    python -m gplite_gb300.selftest M N K [slices] [repeats]

computes C = C - A B^T for random M x K and N x K operands with the BF16-sliced
tcgen05 GEMM and with the FP64 GEMM (gpgp_mixed_selftest), and prints the
relative difference with the GEMM's launch count, time and BF16 MMA rate from
the library's kernel timers. The first call is a warm-up.

    python -m gplite_gb300.selftest fit|fitgrad N M [fp64|mixed] [repeats]

runs a full GP regression fit, its energy gradient (fitgrad: in the same call)
and a prediction with variance at M points (see fit_pred): the profiling entry
point of the other kernels.
"""
from __future__ import annotations

import ctypes as C
import sys

from . import _lib as L


def run(M, N, K, slices=4, repeats=1):
    lib = L.load()
    ctx = L.default_context(0)
    err = C.c_double(-1.0)
    L.check(lib.gpgp_mixed_selftest(ctx.h, M, N, K, slices, C.byref(err)), ctx.h)
    lib.gpgp_profile_enable(ctx.h, 1)
    for _ in range(repeats):
        L.check(lib.gpgp_mixed_selftest(ctx.h, M, N, K, slices, C.byref(err)), ctx.h)
    n, ms, fl = C.c_int64(), C.c_double(), C.c_double()
    lib.gpgp_kernel_profile_read(ctx.h, 0, C.byref(n), C.byref(ms), C.byref(fl))
    lib.gpgp_profile_enable(ctx.h, 0)
    return dict(rel_err=err.value, launches=n.value, ms_per_launch=ms.value / max(n.value, 1),
                tflops=fl.value / max(ms.value / 1e3, 1e-30) / 1e12)


def fit_pred(n, m, precision="fp64", d=8, repeats=1, fused=False):
    """A full GP regression (matern52 + const, lik_gaussian 0.05) on n seeded points in
    [-1, 1]^d: gp_fit, the energy gradient (fused: in the same call, gpgp_fit_grad)
    and gp_pred with variance at m points, `repeats` times after one warm-up round.
    The profiling entry point of the covariance, Cholesky, solve, gradient and
    prediction kernels."""
    import time

    import numpy as np

    from . import gp as G
    from .objects import cf_const, cf_matern52, lik_gaussian
    rng = np.random.default_rng(11)
    x = rng.uniform(-1, 1, (n, d))
    y = np.sin(2 * x[:, 0]) + x[:, 1] + 0.05 * rng.standard_normal(n)
    xt = rng.uniform(-1, 1, (m, d))
    out = []
    for r in range(repeats + 1):
        t0 = time.perf_counter()
        g = G.gp_fit(G.gp_init([cf_matern52(lscale=0.7), cf_const(1.0)], lik_gaussian(sigma=0.05)), x, y,
                     precision=precision, grad=fused)
        G.gp_energy_grad(g)
        p = G.gp_pred(g, xt, var=True)
        if r:
            out.append(time.perf_counter() - t0)
    return dict(lml=g.fit["log_evidence"], mean0=float(p["mean"][0]), s_per_round=sum(out) / len(out))


def main(argv):
    if argv and argv[0] in ("fit", "fitgrad"):
        n, m = int(argv[1]), int(argv[2])
        prec = argv[3] if len(argv) > 3 else "fp64"
        r = fit_pred(n, m, prec, repeats=int(argv[4]) if len(argv) > 4 else 1, fused=argv[0] == "fitgrad")
        print("%s + pred n %d m %d %s: lml %.12g, %.3f s per round"
              % ("fit and gradient in one call" if argv[0] == "fitgrad" else "fit, gradient",
                 n, m, prec, r["lml"], r["s_per_round"]))
        return 0
    if len(argv) < 3:
        print(__doc__)
        return 2
    M, N, K = (int(v) for v in argv[:3])
    slices = int(argv[3]) if len(argv) > 3 else 4
    repeats = int(argv[4]) if len(argv) > 4 else 1
    r = run(M, N, K, slices, repeats)
    print("M %d N %d K %d slices %d: rel err %.3e, %d launch(es), %.4f ms each, %.1f TFLOP/s BF16 MMA"
          % (M, N, K, slices, r["rel_err"], r["launches"], r["ms_per_launch"], r["tflops"]))
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv[1:]))
