"""
Prism magnetics on the GPU (hg_prism_magnetic) against the oracle
(1e-8 relative + 1e-9 of the largest value, like the gravity parity), the
sample fixture of test/test_prism_magnetic.py:230-270, null prisms and the
component/vector consistency.
"""

import numpy as np
import numpy.testing as npt
import pytest

import harmonica_gb300 as hg

pytestmark = pytest.mark.gpu


def _parity(a, b):
    b = np.asarray(b)
    npt.assert_allclose(a, b, rtol=1e-8, atol=1e-9 * np.abs(b).max())


def test_reference_fixture_against_oracle(gpu_lib, oracle):
    prisms = np.array([[-10, 10, -10, 0, -10, 0], [-10, 0, -10, 10, -20, -10],
                       [5, 15, 5, 15, -15, -5], [-5, 5, -5, 5, -35, -20]], dtype=float)
    mag = (np.array([1.0, -1.0, 3.0, -1.5]), np.array([1.0, -0.5, -1.0, 2.0]),
           np.array([1.0, 2.0, -3.0, -2.0]))
    coords = (np.array([-5, 10, 0, 15.0]), np.array([14, -4, 11, 0.0]), np.array([9, 6, 6, 12.0]))
    b = hg.prism_magnetic(coords, prisms, mag, "b")
    ref = oracle.prism_magnetic(coords, prisms, mag, "b")
    for got, exp in zip(b, ref):
        _parity(got, exp)
    for k, f in enumerate(("b_e", "b_n", "b_u")):
        _parity(hg.prism_magnetic(coords, prisms, mag, f), ref[k])


def test_random_against_oracle(gpu_lib, oracle):
    rng = np.random.default_rng(5)
    m = 700
    w = rng.uniform(-3e3, 3e3, m)
    s = rng.uniform(-3e3, 3e3, m)
    t = rng.uniform(-600, -50, m)
    prisms = np.column_stack([w, w + rng.uniform(20, 600, m), s, s + rng.uniform(20, 600, m),
                              t - rng.uniform(20, 800, m), t])
    mag = tuple(rng.uniform(-2, 2, m) for _ in range(3))
    coords = (rng.uniform(-4e3, 4e3, 400), rng.uniform(-4e3, 4e3, 400), rng.uniform(0, 300, 400))
    b = hg.prism_magnetic(coords, prisms, mag, "b")
    ref = oracle.prism_magnetic(coords, prisms, mag, "b")
    for got, exp in zip(b, ref):
        _parity(got, exp)


def test_null_prisms_and_far_field(gpu_lib):
    coords = ([30.0, -200.0], [-40.0, 80.0], [0.0, 10.0])
    prism = [-1, 1, -1, 1, -1001, -999]
    full = hg.prism_magnetic(coords, [prism, [0, 0, -1, 1, -5, -1], prism],
                             ([1.0, 5.0, 0.0], [2.0, 5.0, 0.0], [3.0, 5.0, 0.0]), "b")
    single = hg.prism_magnetic(coords, [prism], ([1.0], [2.0], [3.0]), "b")
    for a, c in zip(full, single):
        npt.assert_allclose(a, c, rtol=1e-13)
    r = np.array([30.0, -40.0, 1000.0])
    m = np.array([1.0, 2.0, 3.0]) * 8.0
    R = np.linalg.norm(r)
    dip = 1e-7 * (3 * r * np.dot(m, r) / R ** 5 - m / R ** 3) * 1e9
    npt.assert_allclose([c[0] for c in single], dip, rtol=1e-4)


def test_parallel_and_progressbar_flags(gpu_lib):
    """test/test_prism_magnetic.py: results with parallel=False and with the
    progress bar equal the defaults (both flags are accepted; the GPU path
    has one evaluation order)."""
    rng = np.random.default_rng(8)
    m = 50
    w = rng.uniform(-500, 500, m)
    s = rng.uniform(-500, 500, m)
    t = rng.uniform(-300, -20, m)
    prisms = np.column_stack([w, w + rng.uniform(20, 200, m), s, s + rng.uniform(20, 200, m),
                              t - rng.uniform(20, 200, m), t])
    mag = tuple(rng.uniform(-2, 2, m) for _ in range(3))
    coords = (rng.uniform(-800, 800, 90), rng.uniform(-800, 800, 90), rng.uniform(0, 100, 90))
    for f in ("b_e", "b_n", "b_u"):
        base = hg.prism_magnetic(coords, prisms, mag, f)
        npt.assert_array_equal(hg.prism_magnetic(coords, prisms, mag, f, parallel=False), base)
        npt.assert_array_equal(hg.prism_magnetic(coords, prisms, mag, f, progressbar=True), base)
