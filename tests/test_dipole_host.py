"""
Dipoles on the CPU: the oracle against the dipole's physics (on-axis and
equatorial fields, and the far field of a uniformly magnetized prism from
the prism-magnetic oracle) and the host checks of harmonica_gb300.dipole
mirroring test/test_dipole.py.
"""

import re

import numpy as np
import numpy.testing as npt
import pytest

from harmonica_gb300 import dipole as hd
from oracle import dipole_oracle, prism_oracle


def test_oracle_axis_and_equator():
    """On the axis b = mu0/(4 pi) 2 m / r^3, on the equator -mu0/(4 pi) m / r^3."""
    m, r = 1e9, 500.0
    b = dipole_oracle.dipole_magnetic(([0.0, r], [0.0, 0.0], [r, 0.0]), ([0.0], [0.0], [0.0]),
                                      ([0.0], [0.0], [m]))
    npt.assert_allclose(b[2], [2e-7 * m / r**3 * 1e9, -1e-7 * m / r**3 * 1e9], rtol=1e-14)
    npt.assert_allclose(b[0], [0.0, 0.0], atol=1e-20)


def test_oracle_matches_prism_far_field():
    """A small uniformly magnetized prism far away is a dipole of moment M V."""
    prism = np.array([[-5.0, 5.0, -5.0, 5.0, -105.0, -95.0]])
    mag = (np.array([1.0]), np.array([-0.5]), np.array([2.0]))
    pts = (np.array([300.0, -200.0, 50.0]), np.array([100.0, 400.0, -350.0]),
           np.array([250.0, 300.0, 500.0]))
    vol = 1000.0
    got = dipole_oracle.dipole_magnetic(pts, ([0.0], [0.0], [-100.0]),
                                        tuple(vol * m for m in mag))
    for k, comp in enumerate(("b_e", "b_n", "b_u")):
        ref = prism_oracle.prism_magnetic(pts, prism, mag, comp)
        npt.assert_allclose(got[k], ref, rtol=2e-3)



def test_oracle_poisson_relation_with_point_mass_tensor():
    """A dipole's field is mu0/(4 pi G) times the gravity tensor of a unit
    point mass at the dipole contracted with the moment (the tensor from the
    point-mass oracle; g_ez and g_nz are easting/northing-downward)."""
    dipoles = (np.array([0.0, 120.0, -80.0]), np.array([0.0, -40.0, 60.0]),
               np.array([-100.0, -300.0, -50.0]))
    moments = (np.array([2e6, -1e6, 5e5]), np.array([-3e5, 4e6, 1e6]),
               np.array([1e6, 2e6, -3e6]))
    pts = (np.array([300.0, -200.0, 50.0, 10.0]), np.array([100.0, 400.0, -350.0, 20.0]),
           np.array([250.0, 300.0, 500.0, -20.0]))
    expected = np.zeros((3, 4))
    for j in range(3):
        src = tuple([c[j]] for c in dipoles)
        g = {f: np.asarray(prism_oracle.point_gravity(pts, src, [1.0], f))
             for f in ("g_ee", "g_nn", "g_zz", "g_en", "g_ez", "g_nz")}
        tensor = np.array([[g["g_ee"], g["g_en"], -g["g_ez"]],
                           [g["g_en"], g["g_nn"], -g["g_nz"]],
                           [-g["g_ez"], -g["g_nz"], g["g_zz"]]])  # Eotvos per kg
        m = np.array([c[j] for c in moments])
        expected += 1e-7 / 6.6743e-11 * np.einsum("ijk,j->ik", tensor, m)
    got = dipole_oracle.dipole_magnetic(pts, dipoles, moments)
    npt.assert_allclose(np.array(got), expected, rtol=1e-12, atol=1e-14 * np.abs(expected).max())

def test_invalid_field():
    """test/test_dipole.py:29-38."""
    msg = re.escape("Invalid field 'Not a valid field'. Please choose one of")
    with pytest.raises(ValueError, match=msg):
        hd.dipole_magnetic((0, 0, 0), (1, 1, 1), (1, 1, 1), field="Not a valid field")


def test_checks_of_moments():
    """test/test_dipole.py:74-110."""
    dipoles = (np.arange(3.0), np.arange(3.0), np.arange(3.0))
    with pytest.raises(ValueError, match="Invalid magnetic moments with '2' elements"):
        hd._check_dipoles_and_magnetic_moments(dipoles, (np.ones(3), np.ones(3)))
    with pytest.raises(ValueError, match=re.escape(
            "Number of elements in magnetic_moments (2) mismatch the number of dipoles (3).")):
        hd._check_dipoles_and_magnetic_moments(dipoles, (np.ones(2), np.ones(2), np.ones(2)))
