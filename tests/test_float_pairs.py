"""
Precision of the packed float-pair distance terms shared by the tesseroid
and point-mass kernels (lean_packed.cuh: p2_diff, p2_norm2, p2_rsqrt),
compiled for the host, against 40-digit mpmath on the same double inputs:
1 / |P - Q| and (P_z - Q_z) / |P - Q|^3 within a few 1e-13 relative for
Earth-centred coordinates (6.4e6 m) at 30 km - 3000 km (measured 1.2e-13
and 2.1e-13), and for survey coordinates up to 1e5 m from the origin within
the 48-bit coordinate rounding, 2^-48 x 1e5 m / d: 4e-11 at d = 10 m,
4e-14 at 10 km (measured 1.6e-11 and 2.9e-11 at 19-25 m) -- the claims of
the kernels' comments.
"""

import ctypes
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "native"))


@pytest.fixture(scope="module")
def pairs():
    import build_host

    lib = ctypes.CDLL(build_host.build())
    dp = ctypes.POINTER(ctypes.c_double)
    lib.host_pairs.argtypes = [ctypes.c_int, ctypes.c_int64, dp, dp, dp, dp, dp]

    def run(kind, p, q):
        p = [np.ascontiguousarray(x, dtype=float) for x in p]
        q = np.ascontiguousarray(np.column_stack(q).ravel(), dtype=float)
        out = np.empty_like(p[0])
        P = lambda x: x.ctypes.data_as(dp)  # noqa: E731
        lib.host_pairs(kind, p[0].size, P(p[0]), P(p[1]), P(p[2]), P(q), P(out))
        return out

    return run


def exact(kind, p, q):
    mpmath = pytest.importorskip("mpmath")  # CPU test: the GPU image has no mpmath
    mpmath.mp.dps = 40
    res = []
    for i in range(p[0].size):
        d = [mpmath.mpf(float(p[k][i])) - mpmath.mpf(float(q[k][i])) for k in range(3)]
        r = mpmath.sqrt(d[0] ** 2 + d[1] ** 2 + d[2] ** 2)
        res.append(float(1 / r if kind == 0 else d[2] / r**3))
    return np.array(res)


def earth_case(rng, n, dmin, dmax):
    r0 = 6371e3
    u = rng.normal(size=(3, n))
    u /= np.linalg.norm(u, axis=0)
    p = r0 * u
    step = rng.normal(size=(3, n))
    step *= rng.uniform(dmin, dmax, n) / np.linalg.norm(step, axis=0)
    return tuple(p), tuple(p - step)


@pytest.mark.parametrize("kind", [0, 1])
def test_earth_centred_pairs(pairs, kind):
    rng = np.random.default_rng(1)
    p, q = earth_case(rng, 300, 3e4, 3e6)
    got = pairs(kind, p, q)
    ref = exact(kind, p, q)
    scale = np.abs(ref) if kind == 0 else 1 / np.linalg.norm(np.subtract(p, q), axis=0) ** 2
    assert np.max(np.abs(got - ref) / scale) < 5e-13


@pytest.mark.parametrize("kind", [0, 1])
def test_survey_pairs(pairs, kind):
    rng = np.random.default_rng(2)
    n = 300
    p = tuple(rng.uniform(-1e5, 1e5, n) for _ in range(3))
    step = rng.normal(size=(3, n))
    step *= 10 ** rng.uniform(1, 5, n) / np.linalg.norm(step, axis=0)
    q = tuple(p[k] - step[k] for k in range(3))
    got = pairs(kind, p, q)
    ref = exact(kind, p, q)
    dist = np.linalg.norm(step, axis=0)
    scale = np.abs(ref) if kind == 0 else 1 / dist**2
    # the bound of the coordinates' 48-bit rounding, with a factor 8 of margin
    assert np.all(np.abs(got - ref) / scale < 8 * 2.0**-48 * 1e5 / dist + 1e-13)
