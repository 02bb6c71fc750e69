"""
Point masses on the GPU (hg_point_forward) against the oracle and the
reference test suite's known answers (test/test_point_gravity.py): sample
potentials, spherical analytic cases, Laplace, finite differences of the
potential, symmetry.  Tolerance vs the oracle: 1e-10 relative + 1e-12 of the
largest value (a short closed form per pair).
"""

import os

import numpy as np
import numpy.testing as npt
import pytest

import harmonica_gb300 as hg

pytestmark = pytest.mark.gpu

CART_FIELDS = ("potential", "g_e", "g_n", "g_z", "g_ee", "g_nn", "g_zz", "g_en", "g_ez", "g_nz",
               "g_ne", "g_ze", "g_zn")


def _random(seed, n_pts, n_obs):
    rng = np.random.default_rng(seed)
    pts = (rng.uniform(-5e3, 5e3, n_pts), rng.uniform(-5e3, 5e3, n_pts),
           rng.uniform(-3e3, -100, n_pts))
    masses = rng.uniform(-1e9, 1e9, n_pts)
    coords = (rng.uniform(-6e3, 6e3, n_obs), rng.uniform(-6e3, 6e3, n_obs),
              rng.uniform(0, 500, n_obs))
    return coords, pts, masses


@pytest.mark.parametrize("field", CART_FIELDS)
def test_cartesian_against_oracle(gpu_lib, oracle, field):
    coords, pts, masses = _random(1, 3000, 700)
    ref = oracle.point_gravity(coords, pts, masses, field)
    res = hg.point_gravity(coords, pts, masses, field)
    npt.assert_allclose(res, ref, rtol=1e-10, atol=1e-12 * np.abs(ref).max())


@pytest.mark.parametrize("field", ("potential", "g_z"))
def test_spherical_against_oracle(gpu_lib, oracle, field):
    rng = np.random.default_rng(2)
    pts = (rng.uniform(-180, 180, 2000), rng.uniform(-80, 80, 2000),
           6.37e6 - rng.uniform(0, 5e4, 2000))
    masses = rng.uniform(1e10, 1e12, 2000)
    coords = (rng.uniform(-180, 180, 300), rng.uniform(-80, 80, 300),
              6.37e6 + rng.uniform(0, 1e4, 300))
    ref = oracle.point_gravity(coords, pts, masses, field, "spherical")
    res = hg.point_gravity(coords, pts, masses, field, coordinate_system="spherical")
    npt.assert_allclose(res, ref, rtol=1e-10, atol=1e-12 * np.abs(ref).max())


def test_reference_sample_potentials(gpu_lib):
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "reference_point_potential.npz"))
    res = hg.point_gravity((g["easting"], g["northing"], g["upward"]), g["point"], g["mass"],
                           "potential")
    npt.assert_allclose(res, g["potential"], rtol=1e-7)


def test_spherical_analytic_cases(gpu_lib):
    """test/test_point_gravity.py:657-710"""
    G = 6.6743e-11
    lon, lat, r = np.meshgrid(np.linspace(-180, 180, 37), np.linspace(-90, 90, 19),
                              np.logspace(1, 8, 5))
    npt.assert_allclose(hg.point_gravity([lon, lat, r], [0.0, 0.0, 0.0], 2.0, "potential",
                                         "spherical"), G * 2.0 / r)
    npt.assert_allclose(hg.point_gravity([lon, lat, r], [0.0, 0.0, 0.0], 2.0, "g_z",
                                         "spherical"), G * 2.0 / r ** 2 * 1e5)
    for lo in (-180.0, 0.0, 95.0):
        for la in (-90.0, 0.0, 45.0):
            for h in (1.0, 1e2, 1e4):
                res = hg.point_gravity([np.array(lo), np.array(la), np.array(3.0 + h)],
                                       [lo, la, 3.0], 2.0, "g_z", "spherical")
                npt.assert_allclose(res, G * 2.0 / h ** 2 * 1e5)


def test_laplace_and_finite_differences(gpu_lib):
    coords, pts, masses = _random(3, 50, 200)
    d = {f: hg.point_gravity(coords, pts, masses, f) for f in ("g_ee", "g_nn", "g_zz")}
    npt.assert_allclose(d["g_ee"] + d["g_nn"], -d["g_zz"], rtol=1e-9,
                        atol=1e-9 * np.abs(d["g_zz"]).max())
    h = 1e-3
    e, n, u = coords
    fd = (hg.point_gravity((e, n, u + h), pts, masses, "potential")
          - hg.point_gravity((e, n, u - h), pts, masses, "potential")) / (2 * h)
    npt.assert_allclose(-fd * 1e5, hg.point_gravity(coords, pts, masses, "g_z"), rtol=1e-5)


def test_many_chunks_and_empty(gpu_lib, oracle):
    coords, pts, masses = _random(4, 20000, 5)
    npt.assert_allclose(hg.point_gravity(coords, pts, masses, "g_z"),
                        oracle.point_gravity(coords, pts, masses, "g_z"), rtol=1e-10)
    assert hg.point_gravity((np.zeros(0),) * 3, pts, masses, "g_z").shape == (0,)
    npt.assert_array_equal(hg.point_gravity(coords, ([], [], []), [], "g_z"), np.zeros(5))


@pytest.mark.parametrize("system", ("cartesian", "spherical"))
def test_parallel_flag(gpu_lib, system):
    """test/test_point_gravity.py (cartesian and spherical parallel tests):
    parallel=False gives the default's results."""
    if system == "cartesian":
        coords, pts, masses = _random(6, 200, 150)
    else:
        rng = np.random.default_rng(6)
        pts = (rng.uniform(-10, 10, 200), rng.uniform(-10, 10, 200),
               6.371e6 - rng.uniform(1e3, 5e4, 200))
        masses = rng.uniform(-1e9, 1e9, 200)
        coords = (rng.uniform(-12, 12, 150), rng.uniform(-12, 12, 150),
                  6.371e6 + rng.uniform(0, 1e3, 150))
    for f in ("potential", "g_z"):
        base = hg.point_gravity(coords, pts, masses, f, coordinate_system=system)
        npt.assert_array_equal(
            hg.point_gravity(coords, pts, masses, f, coordinate_system=system, parallel=False),
            base)
