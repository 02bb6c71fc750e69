"""
Magnetic field of dipoles on the GPU (hg_dipole_magnetic through
harmonica_gb300.dipole_magnetic) against the numpy oracle; FP64 with the
FP32-seeded reciprocal square root (<= 2 ulp), so rtol 1e-12.
"""

import numpy as np
import numpy.testing as npt
import pytest

pytest.importorskip("torch")

from harmonica_gb300 import dipole_magnetic  # noqa: E402
from oracle import dipole_oracle  # noqa: E402

pytestmark = pytest.mark.gpu


def case(seed, n_points, n_dipoles):
    rng = np.random.default_rng(seed)
    coords = (rng.uniform(-5e3, 5e3, n_points), rng.uniform(-5e3, 5e3, n_points),
              rng.uniform(0, 500, n_points))
    dipoles = (rng.uniform(-5e3, 5e3, n_dipoles), rng.uniform(-5e3, 5e3, n_dipoles),
               rng.uniform(-3e3, -100, n_dipoles))
    moments = tuple(rng.normal(0, 1e9, n_dipoles) for _ in range(3))
    return coords, dipoles, moments


@pytest.mark.parametrize("field", ["b_e", "b_n", "b_u"])
def test_components_vs_oracle(field):
    coords, dipoles, moments = case(0, 500, 300)
    got = dipole_magnetic(coords, dipoles, moments, field=field)
    ref = dipole_oracle.dipole_magnetic(coords, dipoles, moments)[("b_e", "b_n", "b_u").index(field)]
    npt.assert_allclose(got, ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())


def test_vector_many_dipoles_chunked():
    """Enough dipoles for chunk partials (the three rows reduced together)."""
    coords, dipoles, moments = case(1, 300, 20000)
    b = dipole_magnetic(coords, dipoles, moments, field="b")
    ref = dipole_oracle.dipole_magnetic(coords, dipoles, moments)
    for got, exp in zip(b, ref, strict=True):
        npt.assert_allclose(got, exp, rtol=1e-11, atol=1e-12 * np.abs(exp).max())


def test_shapes_and_components_consistent():
    """test/test_dipole.py:95-110: 'b' equals the three components; grid shapes."""
    _, dipoles, moments = case(2, 1, 50)
    e, n = np.meshgrid(np.linspace(-4e3, 4e3, 7), np.linspace(-3e3, 3e3, 5))
    coords = (e, n, np.full(e.shape, 200.0))
    b = dipole_magnetic(coords, dipoles, moments, field="b")
    for k, f in enumerate(("b_e", "b_n", "b_u")):
        comp = dipole_magnetic(coords, dipoles, moments, field=f)
        assert comp.shape == e.shape
        npt.assert_allclose(b[k], comp, rtol=1e-13)


def test_disable_checks():
    """test/test_dipole.py:41-55: the checks can be skipped on valid input."""
    coords, dipoles, moments = case(3, 20, 10)
    a = dipole_magnetic(coords, dipoles, moments, field="b_u")
    b = dipole_magnetic(coords, dipoles, moments, field="b_u", disable_checks=True)
    npt.assert_array_equal(a, b)
