"""
CPU oracle for the magnetic field of dipoles — TEST INFRASTRUCTURE ONLY
(tests/ may import it; the product never does).

numpy restatement of harmonica ``src/harmonica/_forward/dipole.py:292-360``
with the closed form of a point dipole (choclo.dipole, third-party, absent
here: the textbook field, b = mu0/(4 pi) (3 (m . r) r / |r|^5 - m / |r|^3)
with r = point - dipole), in nT.
"""

import numpy as np

MU0_OVER_4PI = 1e-7


def dipole_magnetic(coordinates, dipoles, magnetic_moments):
    """(b_e, b_n, b_u) in nT at the points (1-D arrays)."""
    p = np.stack([np.ravel(np.asarray(c, dtype=np.float64)) for c in coordinates[:3]])
    q = np.stack([np.ravel(np.asarray(c, dtype=np.float64)) for c in dipoles[:3]])
    m = np.stack([np.ravel(np.asarray(c, dtype=np.float64)) for c in magnetic_moments[:3]])
    r = p[:, :, None] - q[:, None, :]  # (3, n_points, n_dipoles)
    l2 = np.sum(r * r, axis=0)
    mdr = np.einsum("ij,ikj->kj", m, r)
    b = (3 * mdr * r - m[:, None, :] * l2) / l2**2.5
    return tuple(MU0_OVER_4PI * 1e9 * b[k].sum(axis=1) for k in range(3))
