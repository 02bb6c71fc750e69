"""
The FP64 elementary functions of lean_math.cuh (compiled for the host)
against numpy/mpmath: sqrt, division and log within 1 ulp, log of a quotient
within 2e-16 absolute per unit of |log|, the unwrapped argument within
2.5e-14 absolute (1e-13 relative for small angles: its quotient and
arctangent run on float pairs) -- including special values that take the
generic path.
"""

import ctypes
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "native"))


@pytest.fixture(scope="module")
def lean():
    import build_host

    lib = ctypes.CDLL(build_host.build())
    dp = ctypes.POINTER(ctypes.c_double)
    lib.host_lean.argtypes = [ctypes.c_int, ctypes.c_int64, dp, dp, dp, dp, dp]

    def run(kind, a, b=None, c=None, d=None):
        a = np.ascontiguousarray(a, dtype=float)
        b, c, d = (np.ascontiguousarray(x if x is not None else np.ones_like(a), dtype=float)
                   for x in (b, c, d))
        out = np.empty_like(a)
        P = lambda x: x.ctypes.data_as(dp)  # noqa: E731
        lib.host_lean(kind, a.size, P(a), P(b), P(c), P(d), P(out))
        return out

    return run


def ulps(x, ref):
    return np.abs(x - ref) / np.spacing(np.abs(ref))


def test_sqrt_div_log(lean):
    rng = np.random.default_rng(0)
    x = np.exp(rng.uniform(-200, 200, 200_000))
    y = np.exp(rng.uniform(-200, 200, 200_000))
    assert ulps(lean(0, x), np.sqrt(x)).max() <= 1.0
    assert ulps(lean(1, y, x), y / x).max() <= 1.0
    assert ulps(lean(2, x), np.log(x)).max() <= 1.0
    assert ulps(lean(6, x), 1.0 / np.sqrt(x)).max() <= 2.0
    near = 1 + rng.uniform(-1e-3, 1e-3, 100_000)
    rel = np.abs(lean(2, near) - np.log(near)) / np.abs(np.log(near))
    assert rel.max() < 1e-15


def test_special_values_take_generic_path(lean):
    vals = np.array([0.0, -1.0, np.inf, np.nan, 5e-324, 1e-310])
    with np.errstate(all="ignore"):
        np.testing.assert_array_equal(lean(0, vals), np.sqrt(vals))
        np.testing.assert_array_equal(lean(2, vals), np.log(vals))
        np.testing.assert_array_equal(lean(1, np.ones(6), vals), 1.0 / vals)


def test_log_of_quotient(lean):
    mp = pytest.importorskip("mpmath")
    rng = np.random.default_rng(1)
    n = 3000
    p1, p2, q1 = (np.exp(rng.uniform(-60, 60, n)) for _ in range(3))
    q2 = np.where(np.arange(n) % 2 == 0, np.exp(rng.uniform(-60, 60, n)),
                  p1 * p2 / q1 * (1 + rng.uniform(-1e-6, 1e-6, n)))
    got = lean(3, p1, p2, q1, q2)
    got1 = lean(4, p1, None, q1)
    with mp.workdps(40):
        ref = np.array([float(mp.log(mp.mpf(a) * mp.mpf(b) / (mp.mpf(c) * mp.mpf(d))))
                        for a, b, c, d in zip(p1, p2, q1, q2)])
        ref1 = np.array([float(mp.log(mp.mpf(a) / mp.mpf(c))) for a, c in zip(p1, q1)])
    assert np.all(np.abs(got - ref) <= 2e-16 * np.maximum(np.abs(ref), 1.0) * 4)
    assert np.all(np.abs(got1 - ref1) <= 2e-16 * np.maximum(np.abs(ref1), 1.0) * 4)


def test_unwrapped_argument(lean):
    rng = np.random.default_rng(2)
    ang = rng.uniform(-6.2, 6.2, 100_000)
    mag = np.exp(rng.uniform(-50, 50, ang.size))
    est = ang + rng.uniform(-1e-5, 1e-5, ang.size)
    got = lean(5, mag * np.cos(ang), mag * np.sin(ang), est)
    ref = np.arctan2(np.sin(ang), np.cos(ang))
    ref = ref + 2 * np.pi * np.round((ang - ref) / (2 * np.pi))
    # float-pair rotation and arctangent: ~2^-46 absolute
    assert np.abs(got - ref).max() < 2.5e-14
    tiny = rng.uniform(-1, 1, 10_000) * 10.0 ** rng.uniform(-12, -2, 10_000)
    got = lean(5, np.cos(tiny), np.sin(tiny), tiny)
    # float-pair quotient: ~2^-44 relative for small angles
    assert (np.abs(got - np.arctan2(np.sin(tiny), np.cos(tiny))) / np.abs(tiny)).max() < 1e-13
