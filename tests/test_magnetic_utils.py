"""Magnetic vector helpers (the doctest values of src/harmonica/_utils.py)."""

import numpy as np
import numpy.testing as npt

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
