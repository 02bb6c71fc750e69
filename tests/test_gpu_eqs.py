"""
Equivalent sources on the GPU: hg_eqs_jacobian / hg_eqs_predict against the
numpy oracle (1e-14: the reciprocal square root is within 2 ulp), and the
estimators fitted on the data of point masses, with the reference tests'
criteria (test/test_eq_sources_cartesian.py:113-153: the fit reproduces
its data within 1e-3 max|data|; predictions elsewhere).
"""

import numpy as np
import numpy.testing as npt
import pytest

pytest.importorskip("torch")

from harmonica_gb300 import point_gravity  # noqa: E402
from harmonica_gb300.equivalent_sources import (  # noqa: E402
    EquivalentSources,
    EquivalentSourcesSph,
    greens_jacobian,
    greens_predict,
)
from oracle import eqs_oracle  # noqa: E402

pytestmark = pytest.mark.gpu


def cartesian_case(seed=0, n=400):
    rng = np.random.default_rng(seed)
    coords = (rng.uniform(-5e3, 5e3, n), rng.uniform(-5e3, 5e3, n), rng.uniform(0, 300, n))
    pts = (rng.uniform(-5e3, 5e3, 300), rng.uniform(-5e3, 5e3, 300), rng.uniform(-3e3, -500, 300))
    return coords, pts, rng.normal(0, 1e7, 300)


def spherical_case(seed=1, n=300):
    rng = np.random.default_rng(seed)
    r0 = 6371e3
    coords = (rng.uniform(-10, 10, n), rng.uniform(-10, 10, n), r0 + rng.uniform(0, 1e3, n))
    pts = (rng.uniform(-10, 10, 200), rng.uniform(-10, 10, 200), r0 - rng.uniform(5e3, 3e4, 200))
    return coords, pts, rng.normal(0, 1e7, 200)


@pytest.mark.parametrize("spherical", [False, True])
def test_jacobian_and_predict_vs_oracle(spherical):
    coords, pts, coefs = spherical_case() if spherical else cartesian_case()
    jac = greens_jacobian(coords, pts, spherical=spherical)
    ref = eqs_oracle.jacobian(coords, pts, spherical)
    # spherical: the distance formula's 1 - cos(psi) turns last-bit differences
    # of cos into relative ones of up to 2e-16 / (1 - cos(psi)) (~1e-10 here)
    npt.assert_allclose(jac, ref, rtol=1e-9 if spherical else 1e-14)
    pred = greens_predict(coords, pts, coefs, spherical=spherical)
    npt.assert_allclose(pred, eqs_oracle.predict(coords, pts, coefs, spherical),
                        rtol=1e-9 if spherical else 1e-12, atol=1e-12 * np.abs(pred).max())


def test_jacobian_many_rows_and_empty():
    """More than one row block per column tile; empty inputs."""
    rng = np.random.default_rng(4)
    coords = tuple(rng.uniform(-1e3, 1e3, 1037) for _ in range(3))
    pts = (rng.uniform(-1e3, 1e3, 7), rng.uniform(-1e3, 1e3, 7), rng.uniform(-3e3, -2e3, 7))
    npt.assert_allclose(greens_jacobian(coords, pts), eqs_oracle.jacobian(coords, pts),
                        rtol=1e-14)
    assert greens_jacobian(coords, tuple(np.zeros(0) for _ in range(3))).shape == (1037, 0)


def test_equivalent_sources_cartesian_fit():
    """Data of point masses: the fit reproduces them (atol 1e-3 max|data|,
    test/test_eq_sources_cartesian.py:113-130) and predicts the field at
    other points of the survey area."""
    rng = np.random.default_rng(7)
    masses_pts = (rng.uniform(-4e3, 4e3, 20), rng.uniform(-4e3, 4e3, 20),
                  rng.uniform(-2e3, -1e3, 20))
    masses = rng.uniform(1e6, 1e8, 20)
    e, n = np.meshgrid(np.linspace(-5e3, 5e3, 30), np.linspace(-5e3, 5e3, 30))
    coords = (e.ravel(), n.ravel(), np.full(e.size, 100.0))
    data = point_gravity(coords, masses_pts, masses, field="g_z")
    eqs = EquivalentSources().fit(coords, data)
    npt.assert_allclose(eqs.predict(coords), data, atol=1e-3 * np.abs(data).max())
    e2, n2 = np.meshgrid(np.linspace(-4e3, 4e3, 17), np.linspace(-4e3, 4e3, 17))
    other = (e2, n2, np.full(e2.shape, 100.0))
    true = point_gravity(other, masses_pts, masses, field="g_z")
    npt.assert_allclose(eqs.predict(other), true, atol=2e-2 * np.abs(true).max())
    damped = EquivalentSources(damping=1e-6, depth=2e3).fit(coords, data, weights=np.ones(e.size))
    npt.assert_allclose(damped.predict(coords), data, atol=5e-2 * np.abs(data).max())


def test_equivalent_sources_spherical_fit():
    rng = np.random.default_rng(8)
    r0 = 6371e3
    masses_pts = (rng.uniform(-4, 4, 15), rng.uniform(-4, 4, 15), r0 - rng.uniform(2e4, 5e4, 15))
    masses = rng.uniform(1e9, 1e11, 15)
    lon, lat = np.meshgrid(np.linspace(-5, 5, 25), np.linspace(-5, 5, 25))
    coords = (lon.ravel(), lat.ravel(), np.full(lon.size, r0 + 1e3))
    data = point_gravity(coords, masses_pts, masses, field="g_z", coordinate_system="spherical")
    eqs = EquivalentSourcesSph(relative_depth=3e4).fit(coords, data)
    npt.assert_allclose(eqs.predict(coords), data, atol=1e-3 * np.abs(data).max())
