"""
Prism magnetics without a GPU: argument errors of the drop-in
(test/test_prism_magnetic.py:29-225) and the oracle's physics pins (far-field
dipole limit, b = mu0/(4 pi) T M consistent with the gravity tensor).
"""

import numpy as np
import numpy.testing as npt
import pytest

import harmonica_gb300 as hg


def test_errors():
    with pytest.raises(ValueError, match="Invalid field"):
        hg.prism_magnetic([0, 0, 0], [-1, 1, -1, 1, -2, -1], ([1.0], [1.0], [1.0]), "Bx")
    prisms = [[-1, 1, -1, 1, -2, -1], [-1, 1, -1, 1, -4, -3]]
    with pytest.raises(ValueError, match="Invalid magnetization vectors with '2' elements"):
        hg.prism_magnetic([0, 0, 0], prisms, ([1.0, 1.0], [1.0, 1.0]), "b")
    with pytest.raises(ValueError, match=r"Number of magnetization vectors \(3\) mismatch"):
        hg.prism_magnetic([0, 0, 0], prisms, ([1.0] * 3, [1.0] * 3, [1.0] * 3), "b")
    with pytest.raises(ValueError, match="The bottom boundary can't be greater than the top one"):
        hg.prism_magnetic([0, 0, 0], [-1, 1, -1, 1, -1, -2], ([1.0], [1.0], [1.0]), "b_u")


def test_oracle_far_field_dipole(oracle):
    prism = [-1, 1, -1, 1, -1001, -999]
    M = np.array([1.0, 2.0, 3.0])
    rng = np.random.default_rng(0)
    for _ in range(5):
        pt = rng.uniform(-500, 500, 3)
        r = pt - np.array([0.0, 0.0, -1000.0])
        R = np.linalg.norm(r)
        m = M * 8.0
        dip = 1e-7 * (3 * r * np.dot(m, r) / R ** 5 - m / R ** 3) * 1e9
        b = np.array(oracle.prism_magnetic(tuple([x] for x in pt), prism, tuple([x] for x in M),
                                           "b")).ravel()
        npt.assert_allclose(b, dip, rtol=1e-4)


def test_oracle_tensor_relation(oracle):
    """b_u of an upward magnetization equals mu0/(4 pi) * g_zz / (G rho) (outside)."""
    prism = [-100, 120, -80, 60, -500, -200]
    coords = ([10.0, 300.0], [-20.0, 50.0], [100.0, 30.0])
    bu = oracle.prism_magnetic(coords, prism, ([0.0], [0.0], [2.0]), "b_u")
    gzz = oracle.prism_gravity(coords, prism, [1.0], "g_zz")  # Eotvos for rho = 1
    npt.assert_allclose(bu, 1e-7 * 2.0 * gzz / 6.6743e-11, rtol=1e-12)


def test_oracle_poisson_relation_all_components(oracle):
    """Poisson's relation outside the prism: b_i = mu0/(4 pi G rho) sum_j V_ij M_j,
    with V_ij the gravity tensor of the same prism in the (east, north, up)
    frame (g_ez and g_nz are easting/northing-downward, so V_eu = -g_ez,
    V_nu = -g_nz).  Checks every component for a general magnetization at
    points above, beside and below the prism."""
    prism = [-100, 120, -80, 60, -500, -200]
    coords = ([10.0, 300.0, -250.0, 40.0], [-20.0, 50.0, 10.0, 400.0],
              [100.0, 30.0, -350.0, -900.0])
    m = np.array([1.5, -0.7, 2.0])
    g = {f: np.asarray(oracle.prism_gravity(coords, prism, [1.0], f))
         for f in ("g_ee", "g_nn", "g_zz", "g_en", "g_ez", "g_nz")}
    tensor = np.array([[g["g_ee"], g["g_en"], -g["g_ez"]],
                       [g["g_en"], g["g_nn"], -g["g_nz"]],
                       [-g["g_ez"], -g["g_nz"], g["g_zz"]]])  # Eotvos, rho = 1
    expected = 1e-7 / 6.6743e-11 * np.einsum("ijk,j->ik", tensor, m)
    b = oracle.prism_magnetic(coords, prism, tuple([v] for v in m), "b")
    scale = np.abs(expected).max()
    for k, name in enumerate(("b_e", "b_n", "b_u")):
        npt.assert_allclose(b[k], expected[k], rtol=1e-13, atol=1e-15 * scale, err_msg=name)
        single = oracle.prism_magnetic(coords, prism, tuple([v] for v in m), name)
        npt.assert_allclose(single, b[k], rtol=1e-14, atol=0)
