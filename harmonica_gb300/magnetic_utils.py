"""
Magnetic vector helpers used with the magnetic forward models
(``prism_magnetic``, ``dipole_magnetic``): harmonica ``src/harmonica/_utils.py``
``magnetic_angles_to_vec`` (:28-74), ``magnetic_vec_to_angles`` (:77-158) and
``total_field_anomaly`` (:161-210).  Inclination is positive downward from the
horizontal plane, declination from north, positive east; angles in degrees.
Host numpy (elementwise, no all-pairs work).
"""

import numpy as np

__all__ = ["magnetic_angles_to_vec", "magnetic_vec_to_angles", "total_field_anomaly"]


def magnetic_angles_to_vec(intensity, inclination, declination):
    """(easting, northing, upward) components of a vector of the given
    intensity, inclination and declination (degrees)."""
    inc, dec = np.radians(inclination), np.radians(declination)
    return (intensity * np.cos(inc) * np.sin(dec), intensity * np.cos(inc) * np.cos(dec),
            -intensity * np.sin(inc))


def magnetic_vec_to_angles(magnetic_e, magnetic_n, magnetic_u, degrees=True):
    """Intensity, inclination and declination of a magnetic vector."""
    intensity = np.sqrt(magnetic_e**2 + magnetic_n**2 + magnetic_u**2)
    horizontal = np.sqrt(magnetic_e**2 + magnetic_n**2)
    inclination = np.arctan2(-magnetic_u, horizontal)
    declination = np.arctan2(magnetic_e, magnetic_n)
    if degrees:
        inclination, declination = np.degrees(inclination), np.degrees(declination)
    return intensity, inclination, declination


def total_field_anomaly(magnetic_field, inclination, declination):
    """B . F_hat: the anomalous field projected on the unit vector of the
    regional field (inclination, declination in degrees)."""
    b_e, b_n, b_u = (np.asarray(component) for component in magnetic_field)
    f_e, f_n, f_u = magnetic_angles_to_vec(1, inclination, declination)
    return b_e * f_e + b_n * f_n + b_u * f_u
