"""
CPU oracle for the equivalent-source Jacobian and prediction — TEST
INFRASTRUCTURE ONLY (tests/ may import it; the product never does).

numpy restatement of harmonica ``src/harmonica/_equivalent_sources``:
``jacobian`` and ``predict`` (utils.py:54-96) with ``greens_func_cartesian``
(cartesian.py:635-644: 1 / distance_cartesian) and ``greens_func_spherical``
(spherical.py:413-424: 1 / distance_spherical, utils.py:122-201 of
_forward).  Pinned to the reference: tests/golden/reference_eqs.npz holds
the outputs of the reference's own loops (make_eqs_golden.py), which the
Jacobians here reproduce bit for bit.
"""

import numpy as np


def greens_cartesian(coordinates, points):
    e, n, u = (np.ravel(np.asarray(c, dtype=np.float64))[:, None] for c in coordinates[:3])
    pe, pn, pu = (np.ravel(np.asarray(c, dtype=np.float64))[None, :] for c in points[:3])
    return 1 / np.sqrt((e - pe) ** 2 + (n - pn) ** 2 + (u - pu) ** 2)


def greens_spherical(coordinates, points):
    lon, lat, r = (np.ravel(np.asarray(c, dtype=np.float64))[:, None] for c in coordinates[:3])
    plon, plat, pr = (np.ravel(np.asarray(c, dtype=np.float64))[None, :] for c in points[:3])
    lon, lat, plon, plat = np.radians(lon), np.radians(lat), np.radians(plon), np.radians(plat)
    cospsi = np.sin(plat) * np.sin(lat) + np.cos(plat) * np.cos(lat) * np.cos(plon - lon)
    return 1 / np.sqrt((r - pr) ** 2 + 2 * r * pr * (1 - cospsi))


def jacobian(coordinates, points, spherical=False):
    return (greens_spherical if spherical else greens_cartesian)(coordinates, points)


def predict(coordinates, points, coefs, spherical=False):
    return jacobian(coordinates, points, spherical) @ np.ravel(np.asarray(coefs, dtype=np.float64))
