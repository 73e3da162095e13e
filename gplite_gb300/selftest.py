"""Self-test of the sliced tensor-core GEMM on the local GPU.

    python -m gplite_gb300.selftest M N K [slices] [repeats]

computes C = C - A B^T for random M x K and N x K operands with the BF16-sliced
tcgen05 GEMM and with the FP64 GEMM (gpgp_mixed_selftest), and prints the
relative difference with the GEMM's launch count, time and BF16 MMA rate from
the library's kernel timers. The first call is a warm-up.
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


def main(argv):
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
