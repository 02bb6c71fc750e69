"""
CPU oracle for the tesseroid gravity forward model — TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import this module; the product package never does.

numpy glue around the C restatement in ``tesseroid_oracle.c``:

* ``glq_nodes_weights``: ``src/harmonica/_forward/_tesseroid_utils.py:118-146``
  (numpy's ``leggauss`` for the degrees (2, 2, 2) of
  ``tesseroid_gravity.py:29``);
* ``longitude_continuity``: ``_tesseroid_utils.py:471-500``;
* ``discard_null_tesseroids``: ``_tesseroid_utils.py:503-538``;
* ``tesseroid_gravity``: ``src/harmonica/_forward/tesseroid_gravity.py:35-216``
  for constant densities (the adaptive discretisation and quadrature run in
  C; sign flip and mGal conversion of :209-215 here).

The reference's input validation (``_check_tesseroids``, the points-inside
test) is host logic of the product and is tested there; the oracle trusts
its inputs, except that it applies the longitude continuity the reference
applies while checking.
"""

import numpy as np
from numpy.polynomial.legendre import leggauss

from .prism_oracle import _f64, _load, _ptr

GLQ_DEGREES = (2, 2, 2)
STACK_SIZE = 100
MAX_DISCRETIZATIONS = 100000
DISTANCE_SIZE_RATII = {"potential": 1, "g_z": 2.5}
FIELD_CODES = {"potential": 0, "g_z": 1}


def glq_nodes_weights(glq_degrees=GLQ_DEGREES):
    """Unscaled nodes and weights, flattened as [lon, lat, rad] x 2."""
    nodes, weights = [], []
    for degree in glq_degrees:
        x, w = leggauss(degree)
        nodes.append(x)
        weights.append(w)
    return _f64(np.concatenate(nodes)), _f64(np.concatenate(weights))


def longitude_continuity(tesseroids):
    """Move w > e tesseroids to [-180, 180) (copy)."""
    tesseroids = np.array(tesseroids, dtype=np.float64)
    west, east = tesseroids[:, 0], tesseroids[:, 1]
    change = west > east
    east[change] = ((east[change] + 180) % 360) - 180
    west[change] = ((west[change] + 180) % 360) - 180
    return tesseroids


def discard_null_tesseroids(tesseroids, density):
    west, east, south, north, bottom, top = tuple(tesseroids[:, i] for i in range(6))
    null = (west == east) | (south == north) | (bottom == top)
    null[density == 0] = True
    keep = np.logical_not(null)
    return tesseroids[keep, :], density[keep]


def tesseroid_dimensions(tesseroid):
    out = np.zeros(3)
    _load().oracle_tesseroid_dimensions(_ptr(_f64(tesseroid)), _ptr(out))
    return tuple(out)


def distance_tesseroid_point(point, tesseroid):
    return _load().oracle_distance_tesseroid_point(
        float(point[0]), float(point[1]), float(point[2]), _ptr(_f64(tesseroid))
    )


def adaptive_discretization(point, tesseroid, distance_size_ratio, radial_discretization=False,
                            stack_size=STACK_SIZE, max_discretizations=MAX_DISCRETIZATIONS):
    """Small tesseroids of one pair in the reference's order, shape (n, 6)."""
    lib = _load()
    pt, t = _f64(point), _f64(tesseroid)
    cap = 4096
    while True:
        out = np.zeros((cap, 6))
        n = lib.oracle_adaptive_discretization(
            _ptr(pt), _ptr(t), float(distance_size_ratio), int(radial_discretization),
            int(stack_size), int(max_discretizations), _ptr(out), cap,
        )
        if n == -1:
            raise OverflowError("Stack Overflow. Try to increase the stack size.")
        if n == -2:
            raise OverflowError(
                "Exceeded maximum discretizations. Please increase the MAX_DISCRETIZATIONS."
            )
        if n <= cap:
            return out[:n]
        cap = int(n)


def tesseroid_gravity(coordinates, tesseroids, density, field,
                      radial_adaptive_discretization=False, disable_checks=False,
                      parallel=True, trig_perturbation=False, node_density=None):
    """Reference result (potential J/kg, g_z mGal).  ``density``: one value
    per tesseroid; or ``node_density`` (M, 2): the density at the two radial
    nodes of each tesseroid, as gauss_legendre_quadrature_variable_density
    evaluates a density function (2D discretization only; the tesseroids are
    then used as given, without the null discard, like the reference's
    variable-density loop).  ``trig_perturbation`` moves every cos/sin/acos by
    -1, 0 or +1 ulp (a conditioning probe: how much the result depends on the
    libm)."""
    if field not in FIELD_CODES:
        msg = f"Gravitational field {field} not recognized"
        raise ValueError(msg)
    cast = np.broadcast(*coordinates[:3])
    lon, lat, rad = (_f64(np.broadcast_to(c, cast.shape).ravel()) for c in coordinates[:3])
    tess = np.atleast_2d(np.asarray(tesseroids, dtype=np.float64))
    if not disable_checks and (tess[:, 0] > tess[:, 1]).any():
        tess = longitude_continuity(tess)
    if node_density is not None:
        if radial_adaptive_discretization:
            raise ValueError("node densities need the 2D discretization")
        rho = _f64(np.asarray(node_density, dtype=np.float64).reshape(-1, 2))
        tess = _f64(tess)
    else:
        rho = np.atleast_1d(np.asarray(density, dtype=np.float64)).ravel()
        tess, rho = discard_null_tesseroids(tess, rho)
        tess, rho = _f64(tess), _f64(rho)
    nodes, weights = glq_nodes_weights()
    result = np.zeros(lon.size)
    lib = _load()
    lib.oracle_set_trig_perturbation(int(bool(trig_perturbation)))
    try:
        rc = lib.oracle_tesseroid_gravity(
            FIELD_CODES[field], int(radial_adaptive_discretization), lon.size, _ptr(lon),
            _ptr(lat), _ptr(rad), tess.shape[0], _ptr(tess), _ptr(rho),
            int(node_density is not None), _ptr(nodes), _ptr(weights), _ptr(result),
            int(parallel),
        )
    finally:
        lib.oracle_set_trig_perturbation(0)
    if rc == 1:
        raise OverflowError("Stack Overflow. Try to increase the stack size.")
    if rc == 2:
        raise OverflowError(
            "Exceeded maximum discretizations. Please increase the MAX_DISCRETIZATIONS."
        )
    if field == "g_z":
        result *= -1
        result *= 1e5
    return result.reshape(cast.shape)


def spherical_shell(top, bottom, density, radius):
    """Closed-form potential and g_z of a homogeneous spherical shell, the
    analytic check of test/test_tesseroid.py:662-680."""
    g = 6.6743e-11
    potential = 4 / 3 * np.pi * g * density * (top**3 - bottom**3) / radius
    return {"potential": potential, "g_z": 1e5 * potential / radius}


__all__ = [
    "DISTANCE_SIZE_RATII",
    "MAX_DISCRETIZATIONS",
    "STACK_SIZE",
    "adaptive_discretization",
    "discard_null_tesseroids",
    "distance_tesseroid_point",
    "glq_nodes_weights",
    "longitude_continuity",
    "spherical_shell",
    "tesseroid_dimensions",
    "tesseroid_gravity",
]
