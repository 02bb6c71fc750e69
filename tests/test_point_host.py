"""
Point masses without a GPU: the oracle against the reference's own sample
potentials (test/data/sample_point_gravity.csv via tests/golden) and the
drop-in's argument errors (test/test_point_gravity.py:41-113).
"""

import os

import numpy as np
import numpy.testing as npt
import pytest

import harmonica_gb300 as hg


def test_oracle_against_reference_samples(oracle):
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "reference_point_potential.npz"))
    res = oracle.point_gravity((g["easting"], g["northing"], g["upward"]), g["point"], g["mass"],
                               "potential")
    npt.assert_allclose(res, g["potential"], rtol=1e-7)


def test_oracle_spherical_analytic(oracle):
    G = 6.6743e-11
    lon, lat, r = np.meshgrid(np.linspace(-180, 180, 7), np.linspace(-90, 90, 5),
                              np.logspace(1, 8, 3))
    for field, sol in (("potential", G * 2.0 / r), ("g_z", G * 2.0 / r ** 2 * 1e5)):
        npt.assert_allclose(oracle.point_gravity([lon, lat, r], [0.0, 0.0, 0.0], 2.0, field,
                                                 "spherical"), sol, rtol=1e-12)


def test_errors():
    with pytest.raises(ValueError, match="Coordinate system geodetic not recognized"):
        hg.point_gravity([0, 0, 0], [0, 0, -1], [1.0], "g_z", coordinate_system="geodetic")
    for field in ("g_n", "g_e"):
        with pytest.raises(NotImplementedError):
            hg.point_gravity([0, 0, 1], [0, 0, 0], [1.0], field, coordinate_system="spherical")
    for system in ("cartesian", "spherical"):
        with pytest.raises(ValueError, match="Gravitational field 'this-field' not recognized"):
            hg.point_gravity([0, 0, 1], [0, 0, 0], [1.0], "this-field", coordinate_system=system)
    msg = r"Number of elements in masses \([0-9]+\) mismatch the number of points \([0-9]+\)"
    with pytest.raises(ValueError, match=msg):
        hg.point_gravity([0, 0, 250], [[-10, 0], [0, 0], [-100, -10]], [1000, 2000, 3000],
                         "potential")


def test_oracle_spherical_matches_reference_golden(oracle):
    """Spherical potential and g_z against harmonica's own point_gravity run
    from the reference sources (tests/golden/make_point_golden.py; its
    spherical kernels are harmonica code), masses right below, near and far
    from the points: measured agreement 2.5e-16."""
    import os

    g = np.load(os.path.join(os.path.dirname(__file__), "golden",
                             "reference_point_spherical.npz"))
    for field in ("potential", "g_z"):
        got = oracle.point_gravity(tuple(g["coordinates"]), tuple(g["points"]), g["masses"],
                                   field, coordinate_system="spherical")
        npt.assert_allclose(got, g[field], rtol=1e-14, atol=0)
