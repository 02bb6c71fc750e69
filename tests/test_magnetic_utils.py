"""Magnetic vector helpers: the doctest values of src/harmonica/_utils.py,
known directions (axes, diagonals, tiny vectors) and the total field anomaly
with lists, arrays and per-point directions."""

import numpy as np
import numpy.testing as npt
import pytest

from harmonica_gb300.magnetic_utils import (
    magnetic_angles_to_vec,
    magnetic_vec_to_angles,
    total_field_anomaly,
)


def test_angles_to_vec_and_back():
    e, n, u = magnetic_angles_to_vec(3.0, 45.0, 45.0)
    npt.assert_allclose([e, n, u], [1.5, 1.5, -2.121], atol=5e-4)
    intensity, inc, dec = magnetic_vec_to_angles(1.5, 1.5, -2.12132)
    npt.assert_allclose([intensity, inc, dec], [3.0, 45.0, 45.0], atol=1e-4)
    rng = np.random.default_rng(0)
    vec = rng.normal(size=(3, 50))
    back = magnetic_angles_to_vec(*magnetic_vec_to_angles(*vec))
    npt.assert_allclose(back, vec, rtol=1e-12, atol=1e-14)
    _, inc_r, dec_r = magnetic_vec_to_angles(*vec, degrees=False)
    npt.assert_allclose(np.degrees(inc_r), magnetic_vec_to_angles(*vec)[1])


def test_total_field_anomaly():
    """A field parallel to the regional one projects to its intensity, a
    perpendicular one to zero."""
    b = magnetic_angles_to_vec(50.0, 30.0, -20.0)
    npt.assert_allclose(total_field_anomaly(b, 30.0, -20.0), 50.0, rtol=1e-14)
    f_hat = np.array(magnetic_angles_to_vec(1.0, 30.0, -20.0))
    other = np.array([0.3, -1.2, 0.7])
    perp = other - (other @ f_hat) * f_hat
    npt.assert_allclose(total_field_anomaly(perp, 30.0, -20.0), 0.0, atol=1e-14)


# unit-intensity directions and their (easting, northing, upward) vectors:
# inclination positive downward, declination clockwise from north
_DIRECTIONS = [
    ((1.0, 45.0, 45.0), (0.5, 0.5, -np.sqrt(0.5))),
    ((1.0, -45.0, 45.0), (0.5, 0.5, np.sqrt(0.5))),
    ((1.0, 45.0, -45.0), (-0.5, 0.5, -np.sqrt(0.5))),
    ((1.0, 90.0, 0.0), (0.0, 0.0, -1.0)),
    ((1.0, 0.0, 90.0), (1.0, 0.0, 0.0)),
    ((1.0, 0.0, 0.0), (0.0, 1.0, 0.0)),
    ((1e-13, 90.0, 0.0), (0.0, 0.0, -1e-13)),
    ((1e-13, 0.0, 90.0), (1e-13, 0.0, 0.0)),
    ((1e-13, 0.0, 0.0), (0.0, 1e-13, 0.0)),
]


@pytest.mark.parametrize(("angles", "vector"), _DIRECTIONS)
def test_known_directions(angles, vector):
    """Angles -> vector and vector -> angles (degrees and radians) on the
    axes, the diagonals and vectors of 1e-13 intensity."""
    npt.assert_allclose(magnetic_angles_to_vec(*angles), vector, rtol=1e-12, atol=1e-15)
    intensity, inc, dec = angles
    npt.assert_allclose(magnetic_vec_to_angles(*vector), (intensity, inc, dec), rtol=1e-12,
                        atol=1e-12)
    npt.assert_allclose(magnetic_vec_to_angles(*vector, degrees=False),
                        (intensity, np.radians(inc), np.radians(dec)), rtol=1e-12, atol=1e-14)


def test_known_directions_as_arrays():
    angles = np.array([a for a, _ in _DIRECTIONS]).T
    vectors = np.array([v for _, v in _DIRECTIONS]).T
    npt.assert_allclose(magnetic_angles_to_vec(*angles), vectors, rtol=1e-12, atol=1e-15)
    npt.assert_allclose(magnetic_vec_to_angles(*vectors), angles, rtol=1e-12, atol=1e-12)
    npt.assert_allclose(magnetic_angles_to_vec(*magnetic_vec_to_angles(*vectors)), vectors,
                        rtol=1e-12, atol=1e-15)


@pytest.mark.parametrize(("inc", "dec", "component"),
                         [(0.0, 90.0, 0), (0.0, 0.0, 1), (-90.0, 0.0, 2)])
def test_tfa_along_axes(inc, dec, component):
    """A regional field along an axis picks that component of B, for B given
    as plain lists of floats or of per-point values."""
    b = [30.0, -40.0, 50.0]
    npt.assert_allclose(total_field_anomaly(b, inc, dec), b[component], atol=1e-12)
    b_arrays = [[20, -30, -40, 50], [-60, 70, -80, 10], [21, -31, 41, -51]]
    npt.assert_allclose(total_field_anomaly(b_arrays, inc, dec), b_arrays[component],
                        atol=1e-12)


def test_tfa_per_point_directions():
    """Inclination and declination given per point (lists)."""
    be, bn, bu = [20.0, -30.0, -40.0, 50.0], [-60.0, 70.0, -80.0, 10.0], [21.0, -31.0, 41.0, -51.0]
    tfa = total_field_anomaly([be, bn, bu], [0.0, 0.0, 45.0, -90.0], [90.0, 0.0, 45.0, 0.0])
    expected = [be[0], bn[1], 0.5 * be[2] + 0.5 * bn[2] - np.sqrt(0.5) * bu[2], bu[3]]
    npt.assert_allclose(tfa, expected, atol=1e-12)
    # a regional field pointing straight down projects -b_u
    npt.assert_allclose(total_field_anomaly([0, 0, -50e3], 90.0, 0.0), 50e3)
