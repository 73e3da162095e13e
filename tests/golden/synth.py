"""Seeded synthetic inputs that every machine reproduces bit for bit.

The golden fixtures freeze oracle outputs on inputs with the workloads' shapes
and distributions. Inputs that only need uniform draws are rebuilt here from
the raw 64-bit stream of numpy's PCG64 bit generator (a fixed algorithm seeded
through SeedSequence), converted to doubles by integer arithmetic, so the
tests rebuild exactly the values the fixtures were made from instead of
storing them. Draws that need transcendental functions (normals, GP draws)
are stored in the fixtures instead, rounded to float32 so that the stored
value is exact.
"""
import numpy as np


def uniform(seed, shape, lo=0.0, hi=1.0):
    """lo + (hi - lo) * u with u = (raw >> 11) * 2^-53 in [0, 1): exact on any machine
    for the power-of-two widths used here."""
    n = int(np.prod(shape))
    raw = np.random.PCG64(seed).random_raw(n)
    u = (raw >> np.uint64(11)).astype(np.float64) * (2.0 ** -53)
    return (lo + (hi - lo) * u).reshape(shape)


# first raw draws of the seeds the fixtures use, and the sum of the C2 inputs: a
# machine whose bit generator or conversion differed would fail check_streams()
# instead of reporting a kernel error
_FIRST_RAW = {20: 0x47b30eebe46aa97a, 22: 0x5dc8e954c570497b, 50: 0xc9948895c805748d,
              51: 0xf143d38462725b3c, 52: 0x9da2a418f6fb8327, 400: 0x32f823c1ca8ca777,
              500: 0x91161420a8e4325e, 600: 0x36a4c3434ad4330d}
_C2_X_SUM = float.fromhex("0x1.57f6746da567cp+8")


def check_streams():
    for seed, v in _FIRST_RAW.items():
        assert int(np.random.PCG64(seed).random_raw(1)[0]) == v, "PCG64 stream differs (seed %d)" % seed
    assert float(c2_inputs()[0].sum()) == _C2_X_SUM, "the C2 inputs differ from the fixture's"


def permutation(seed, n):
    """A permutation of range(n) ordered by raw 64-bit draws."""
    return np.argsort(np.random.PCG64(seed).random_raw(n), kind="stable")


def to_f32_exact(a):
    """Round to the nearest float32, returned as float64 (stored as float32 losslessly)."""
    return np.asarray(a, dtype=np.float32).astype(np.float64)


# ---------------------------------------------------------------------------
# the workloads' inputs (shapes and distributions of the five configurations)
# ---------------------------------------------------------------------------

C2_N, C2_D, C2_M = 16384, 8, 8192
C2_LSCALE, C2_MAGN, C2_CMAGN, C2_SIGMA = 0.7, 1.0, 1.0, 0.05


def c2_inputs(n=C2_N, m=C2_M):
    """x ~ U[-1, 1]^8 (n x 8) and m test points of the same law."""
    return uniform(20, (n, C2_D), -1.0, 1.0), uniform(22, (m, C2_D), -1.0, 1.0)


FITC_N, FITC_M, FITC_D, FITC_MT = 65536, 256, 2, 256


def fitc_inputs():
    """x ~ U[-2, 2]^2 (65536 x 2), 256 inducing inputs chosen at random among x,
    256 test points of the same law."""
    x = uniform(50, (FITC_N, FITC_D), -2.0, 2.0)
    z = x[np.sort(permutation(51, FITC_N)[:FITC_M])]
    xt = uniform(52, (FITC_MT, FITC_D), -2.0, 2.0)
    return x, z, xt


# C4: two problems in every 64-wide size bucket from 64 to 1024
C4_SIZES = [s for b in range(16) for s in (64 * b + 64 - 63 * (b > 0), 64 * b + 64)]


def c4_problem(i, n):
    """Problem i of the C4 sample: d in {1, 2, 3}, sexp or matern32, lscale ~ LogU[0.2, 2],
    sigma ~ U[0.01, 0.3], x ~ U[-2, 2]^d, 128 test points."""
    u = uniform(400 + i, (4,))
    d = 1 + int(u[0] * 3)
    kind = "sexp" if u[1] < 0.5 else "matern32"
    lscale = float(np.exp(np.log(0.2) + u[2] * (np.log(2.0) - np.log(0.2))))
    sigma = float(0.01 + u[3] * 0.29)
    x = uniform(500 + i, (n, d), -2.0, 2.0)
    xt = uniform(600 + i, (128, d), -2.0, 2.0)
    return dict(n=n, d=d, kind=kind, lscale=lscale, sigma=sigma, x=x, xt=xt)
