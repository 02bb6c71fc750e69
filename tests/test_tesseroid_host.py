"""
Tesseroids on the CPU: the oracle against harmonica's own outputs and
analytic solutions, and the host logic of harmonica_gb300.tesseroid (checks,
messages, longitude continuity) mirroring test/test_tesseroid.py of the
reference.
"""

import os
import re

import numpy as np
import numpy.testing as npt
import pytest

from harmonica_gb300 import tesseroid as ht
from oracle import tesseroid_oracle as to

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "reference_tesseroid.npz")
# Earth's mean radius (IUGG, metres)
MEAN_RADIUS = 6371008.8
# test/test_tesseroid.py:45
ACCURACY_THRESHOLD = 1e-3


def _golden():
    return np.load(GOLDEN)


def golden_keys():
    return [str(k) for k in _golden()["names"]]


def golden_case(key):
    g = _golden()
    radial, disable = (bool(v) for v in g[f"{key}_flags"])
    field = "g_z" if key.endswith("g_z") else "potential"
    return (tuple(g[f"{key}_coords"]), g[f"{key}_tesseroids"], g[f"{key}_density"], field,
            radial, disable, g[f"{key}_result"])


@pytest.mark.parametrize("key", golden_keys())
def test_oracle_matches_reference(key):
    """Oracle vs harmonica's tesseroid_gravity run on the same inputs: equal
    up to 1 ulp (numpy's vectorised cos of the point latitudes)."""
    coords, tess, dens, field, radial, disable, expected = golden_case(key)
    got = to.tesseroid_gravity(coords, tess, dens, field, radial_adaptive_discretization=radial,
                               disable_checks=disable)
    npt.assert_allclose(got.ravel(), expected, rtol=1e-14, atol=0)


def test_oracle_small_tesseroids_match_reference():
    """Small tesseroids of one pair in the reference's order
    (test/test_tesseroid.py:642-660), and the stack overflow of the same pair
    with the radial split."""
    g = _golden()
    tess = [-10.0, 10.0, -10.0, 10.0, 1.0, 10.0]
    small = to.adaptive_discretization([0.0, 0.0, 10.0], tess, 10, False)
    npt.assert_array_equal(small, g["split_radial0"])
    assert (small[:, 4] == 1.0).all() and (small[:, 5] == 10.0).all()
    assert g["split_radial1"].shape[0] == 0
    with pytest.raises(OverflowError, match="Stack Overflow"):
        to.adaptive_discretization([0.0, 0.0, 10.0], tess, 10, True)


def test_oracle_overflow_limits():
    """test/test_tesseroid.py:318-336: a stack of 2 and a small-tesseroid
    buffer of 2 both overflow."""
    tess = [-10.0, 10.0, -10.0, 10.0, 0.5, 1.0]
    point = [0.0, 0.0, 1.0]
    with pytest.raises(OverflowError, match="Stack Overflow"):
        to.adaptive_discretization(point, tess, 10, stack_size=2)
    with pytest.raises(OverflowError, match="Exceeded maximum discretizations"):
        to.adaptive_discretization(point, tess, 10, max_discretizations=2)


def test_oracle_distance_tesseroid_point():
    """test/test_tesseroid.py:378-409."""
    lon_p, lat_p, r_p = 0.0, 0.0, MEAN_RADIUS
    d_lon, d_lat, d_radius = 2.0, 2.0, 1.3
    tess = [lon_p - d_lon / 2, lon_p + d_lon / 2, lat_p - d_lat / 2, lat_p + d_lat / 2,
            r_p - d_radius / 2, r_p + d_radius / 2]
    npt.assert_allclose(to.distance_tesseroid_point([lon_p, lat_p, r_p], tess), 0.0)
    npt.assert_allclose(to.distance_tesseroid_point([lon_p, lat_p, r_p + 1.0], tess), 1.0)
    dist = 2 * r_p * np.sin(0.5 * np.radians(3.0))
    npt.assert_allclose(to.distance_tesseroid_point([3.0, lat_p, r_p], tess), dist)
    npt.assert_allclose(to.distance_tesseroid_point([lon_p, 3.0, r_p], tess), dist)


def test_oracle_tesseroid_dimensions():
    """test/test_tesseroid.py:413-420."""
    w, e, s, n, bottom, top = -1.0, 1.0, -1.0, 1.0, 0.5, 1.5
    expected = (top * np.radians(e - w), top * np.radians(n - s), top - bottom)
    npt.assert_allclose(to.tesseroid_dimensions([w, e, s, n, bottom, top]), expected)


def shell(shape, bottom, top):
    longitude = np.linspace(0, 360, shape[0] + 1)
    latitude = np.linspace(-90, 90, shape[1] + 1)
    return np.array([[w, e, s, n, bottom, top]
                     for w, e in zip(longitude[:-1], longitude[1:], strict=True)
                     for s, n in zip(latitude[:-1], latitude[1:], strict=True)])


@pytest.mark.parametrize("field", ["potential", "g_z"])
@pytest.mark.parametrize("thickness", [10, 100, 1e3, 1e4, 1e5])
def test_oracle_spherical_shell_3d(field, thickness):
    """test/test_tesseroid.py:729-770."""
    radius = MEAN_RADIUS + 1e3
    top, bottom = MEAN_RADIUS, MEAN_RADIUS - thickness
    tess = shell((6, 6), bottom, top)
    got = to.tesseroid_gravity([0, 0, radius], tess, np.full(36, 1000.0), field,
                               radial_adaptive_discretization=True)
    npt.assert_allclose(got, to.spherical_shell(top, bottom, 1000, radius)[field],
                        rtol=ACCURACY_THRESHOLD)


@pytest.mark.parametrize("field", ["potential", "g_z"])
def test_oracle_spherical_shell_2d(field):
    """test/test_tesseroid.py:683-726: points on the shell's top surface on a
    10-degree grid, 2D discretisation."""
    radius = MEAN_RADIUS
    lon, lat = np.meshgrid(np.arange(0, 351, 10.0), np.arange(-90, 91, 10.0))
    coords = (lon, lat, np.full(lon.shape, radius))
    for thickness in np.logspace(1, 5, 5):
        tess = shell((12, 6), MEAN_RADIUS - thickness, MEAN_RADIUS)
        got = to.tesseroid_gravity(coords, tess, np.full(72, 1000.0), field)
        expected = to.spherical_shell(MEAN_RADIUS, MEAN_RADIUS - thickness, 1000, radius)[field]
        npt.assert_allclose(got, expected, rtol=ACCURACY_THRESHOLD)


def test_oracle_libm_sensitivity():
    """How much the reference's own result depends on the last bit of its
    libm (every cos/sin/acos moved by -1, 0 or +1 ulp): ~1e-13 far above the
    model, below 1e-8 at 1 km, up to ~1e-3 for points on the face of a 10 m
    shell.  These bound the agreement any other libm (the GPU's) can have
    with the reference; the GPU tests use them as tolerances."""
    def sensitivity(coords, tess, dens, field, radial=False):
        a = to.tesseroid_gravity(coords, tess, dens, field, radial_adaptive_discretization=radial)
        b = to.tesseroid_gravity(coords, tess, dens, field, radial_adaptive_discretization=radial,
                                 trig_perturbation=True)
        return np.max(np.abs(b / a - 1))

    g = _golden()
    far = sensitivity(tuple(g["gallery_g_z_coords"]), g["gallery_g_z_tesseroids"],
                      g["gallery_g_z_density"], "g_z")
    assert far < 1e-11
    near = sensitivity([0, 0, MEAN_RADIUS + 1e3], shell((6, 6), MEAN_RADIUS - 1e3, MEAN_RADIUS),
                       np.full(36, 1000.0), "g_z", radial=True)
    assert near < 1e-8
    lon, lat = np.meshgrid(np.arange(0, 351, 10.0), np.arange(-90, 91, 10.0))
    surface = sensitivity((lon, lat, np.full(lon.shape, MEAN_RADIUS)),
                          shell((12, 6), MEAN_RADIUS - 10.0, MEAN_RADIUS),
                          np.full(72, 1000.0), "g_z")
    assert 1e-5 < surface < ACCURACY_THRESHOLD


# ------------------------------------------------------------ host logic
def test_glq_nodes_weights():
    nodes, weights = ht.glq_nodes_weights((2, 2, 2))
    for x, w in zip(nodes, weights, strict=True):
        x_ref, w_ref = np.polynomial.legendre.leggauss(2)
        npt.assert_array_equal(x, x_ref)
        npt.assert_array_equal(w, w_ref)


def test_longitude_continuity():
    """test/test_tesseroid.py:426-441."""
    t = ht.longitude_continuity(np.atleast_2d([-10, 10, -10, 10, 1, 2]))
    assert t[0, 0] == -10 and t[0, 1] == 10
    t = ht.longitude_continuity(np.atleast_2d([-70, -60, -10, 10, 1, 2]))
    assert t[0, 0] == -70 and t[0, 1] == -60
    t = ht.longitude_continuity(np.atleast_2d([350, 10, -10, 10, 1, 2]))
    assert t[0, 0] == -10 and t[0, 1] == 10


def test_valid_tesseroids_pass():
    """test/test_tesseroid.py:134-152."""
    w, e, s, n, bottom, top = -10, 10, -10, 10, 100, 200
    for t in ([w, e, s, n, bottom, top], [w, w, s, n, bottom, top], [w, e, s, s, bottom, top],
              [w, e, s, n, bottom, bottom], [350, 10, s, n, bottom, top],
              [-70, -60, s, n, bottom, top], [-10, 10, s, n, bottom, top],
              [-150, 150, s, n, bottom, top], [0, 360, s, n, bottom, top],
              [-180, 180, s, n, bottom, top]):
        ht.check_tesseroids(np.atleast_2d(np.array(t, dtype=float)))


def test_invalid_tesseroids_messages():
    """test/test_tesseroid.py:155-221."""
    w, e, s, n, bottom, top = -10, 10, -10, 10, 100, 200

    def bad(t, msg):
        with pytest.raises(ValueError, match=msg):
            ht.check_tesseroids(np.atleast_2d(np.array(t, dtype=float)))

    bad([w, e, n, s, bottom, top], "The south boundary can't be greater than the north one")
    lat_msg = re.escape("The latitudinal boundaries must be inside the [-90, 90] degrees interval")
    for t in ([w, e, s, -100, bottom, top], [w, e, s, 100, bottom, top],
              [w, e, -100, n, bottom, top], [w, e, 100, n, bottom, top]):
        bad(t, lat_msg)
    bad([w, e, s, n, top, bottom], "The bottom radius boundary can't be greater than the top one")
    bad([w, e, s, n, bottom, -1], "The bottom and top radii should be positive or zero")
    bad([w, e, s, n, -1, top], "The bottom and top radii should be positive or zero")
    lon_msg = re.escape(
        "The longitudinal boundaries must be inside the [-180, 360] degrees interval")
    for t in ([-200, e, s, n, bottom, top], [400, e, s, n, bottom, top],
              [w, -200, s, n, bottom, top], [w, 400, s, n, bottom, top]):
        bad(t, lon_msg)
    for t in ([30, 0, s, n, bottom, top], [-60, -70, s, n, bottom, top],
              [300, -150, s, n, bottom, top], [350, 340, s, n, bottom, top]):
        bad(t, "The west boundary can't be greater than the east one")
    bad([-150, 300, s, n, bottom, top],
        "The difference between east and west boundaries cannot be greater than one turn "
        "around the globe")


def test_invalid_field_message():
    """test/test_tesseroid.py:101-109 (raised before any device work)."""
    msg = re.escape("Gravitational field this-field-does-not-exist not recognized")
    with pytest.raises(ValueError, match=msg):
        ht.tesseroid_gravity([0, 0, 250], [-10, 10, -10, 10, 100, 200], 1000,
                             field="this-field-does-not-exist")


def test_inside_message_format():
    """Message of check_points_outside_tesseroids (_tesseroid_utils.py:432-443)."""
    coords = (np.array([0.0]), np.array([0.0]), np.array([150.0]))
    tess = np.array([[-10.0, 10.0, -10.0, 10.0, 100.0, 200.0]])
    msg = ht._inside_message(coords, tess, [(0, 0)])
    assert msg.startswith("Found computation point(s) inside tesseroid(s). "
                          "Computation points must be outside of tesseroids.\n")
    assert " - Computation point '(0.0, 0.0, 150.0)' inside tesseroid " \
           "'(-10.0, 10.0, -10.0, 10.0, 100.0, 200.0)'.\n" in msg


def test_discard_null_tesseroids_oracle():
    """test/test_tesseroid.py:339-371 (the oracle's restatement; the GPU
    path skips the same tesseroids in its prepare kernel)."""
    top, bottom = MEAN_RADIUS, MEAN_RADIUS - 1e3
    tess = np.array([
        [-10, -5, -10, -5, bottom, top], [-10, -5, -5, 0, bottom, top],
        [-10, -10, 0, 5, bottom, top], [-10, -5, 5, 5, bottom, top],
        [-5, 0, -10, -5, top, top], [-5, 0, -5, 0, bottom, top],
        [-5, -5, 5, 5, top, top], [-5, 0, 5, 10, bottom, top],
    ])
    dens = np.array([2400, 0, 2500, 2600, 2700, 2800, 2900, 3000.0])
    t, d = to.discard_null_tesseroids(tess, dens)
    npt.assert_allclose(t, tess[[0, 5, 7]])
    npt.assert_allclose(d, [2400, 2800, 3000])


# ------------------------------------------------------ variable density
GOLDEN_VAR = os.path.join(os.path.dirname(__file__), "golden",
                          "reference_tesseroid_variable.npz")


def _var_golden():
    return np.load(GOLDEN_VAR)


def quadratic_density(radius):
    """test/test_tesseroid_variable_density.py:59-109 (factor 1e-3, vertex
    (3e3, 1900))."""
    return 1e-3 * (radius - 3e3) ** 2 + 1900.0


def linear_shell_density(top, bottom):
    slope = (2500.0 - 3300.0) / (top - bottom)
    constant = 2500.0 - slope * top
    return lambda radius: slope * radius + constant


def exponential_shell_density(top, bottom, b_factor):
    thickness = top - bottom
    a_factor = (3300.0 - 2670.0) / (1 - np.exp(-b_factor))
    constant = 3300.0 - a_factor
    return lambda radius: a_factor * np.exp(-b_factor * (radius - bottom) / thickness) + constant


def variable_density_fn(name):
    top = 6371e3
    return {"linear_shell": linear_shell_density(top, top - 1e3),
            "exponential_shell": exponential_shell_density(top, top - 1e3, 5),
            "single_constant_fn": lambda radius: 2900.0}[name]


def variable_keys():
    return [str(k) for k in _var_golden()["names"]]


def node_densities(tesseroids, fn):
    """The density function at radius_p of the two radial nodes
    (_tesseroid_variable_density.py:87-90), written out independently."""
    x = np.polynomial.legendre.leggauss(2)[0]
    return np.array([[fn(0.5 * (t - b) * x[k] + 0.5 * (t + b)) for k in range(2)]
                     for b, t in tesseroids[:, 4:6]])


def test_density_based_discretization_matches_reference():
    g = _var_golden()
    got = np.array(ht._density_based_discretization((-3, 2, -4, 5, 2e3, 5e3), quadratic_density),
                   dtype=float)
    npt.assert_array_equal(got, g["split_quadratic"])
    # test/test_tesseroid_variable_density.py:223-248: two tesseroids, split at
    # the analytic radius of the largest departure from the chord
    slope = (quadratic_density(5e3) - quadratic_density(2e3)) / 3e3
    npt.assert_allclose(got[0, 4], 0.5 * slope / 1e-3 + 3e3)
    for b in (5, 100):
        t = (0.0, 30.0, 0.0, 30.0, 6371e3 - 1e3, 6371e3)
        got = np.array(ht._density_based_discretization(
            t, exponential_shell_density(t[5], t[4], b)), dtype=float)
        npt.assert_array_equal(got, g[f"split_exponential_{b}"])


def test_density_based_discretization_cases(monkeypatch):
    """test/test_tesseroid_variable_density.py:251-318."""
    tess = [-3, 2, -4, 5, 30, 50]
    assert len(ht._density_based_discretization(tess, lambda r: 3 * r + 2)) == 1
    assert len(ht._density_based_discretization(tess, lambda r: 3)) == 1
    splits = []
    for delta in (1e-3, 1e-2, 1e-1, 1e0):
        monkeypatch.setattr(ht, "DELTA_RATIO", delta)
        splits.append(len(ht._density_based_discretization((-3, 2, -4, 5, 2e3, 5e3),
                                                           quadratic_density)))
    assert (np.diff(splits) < 0).all()


@pytest.mark.parametrize("key", variable_keys())
def test_oracle_variable_density_matches_reference(key):
    """The oracle on the host discretization reproduces harmonica's
    variable-density results bit for bit."""
    g = _var_golden()
    name = key.rsplit("_", 2)[0] if key.endswith("g_z") else key.rsplit("_", 1)[0]
    field = "g_z" if key.endswith("g_z") else "potential"
    fn = variable_density_fn(name)
    tess = ht.density_based_discretization(g[f"{key}_tesseroids"], fn)
    got = to.tesseroid_gravity(tuple(g[f"{key}_coords"]), tess, None, field,
                               node_density=node_densities(tess, fn))
    npt.assert_allclose(got.ravel(), g[f"{key}_result"], rtol=1e-14, atol=0)


def analytic_shell_linear(radius, bottom, top, slope, constant):
    """test/test_tesseroid_variable_density.py:358-372."""
    g = 6.6743e-11
    c = np.pi * g * slope * (top**4 - bottom**4) + 4 / 3 * np.pi * g * constant * (
        top**3 - bottom**3)
    potential = c / radius
    return {"potential": potential, "g_z": 1e5 * potential / radius}


def analytic_shell_exponential(radius, bottom, top, a_factor, b_factor, constant):
    """test/test_tesseroid_variable_density.py:375-409."""
    g = 6.6743e-11
    thickness = top - bottom
    k = b_factor / thickness
    potential = (4 * np.pi * g * a_factor / k**3 / radius * (
        ((bottom * k) ** 2 + 2 * bottom * k + 2)
        - ((top * k) ** 2 + 2 * top * k + 2) * np.exp(-k * thickness))
        + 4 / 3 * np.pi * g * constant * (top**3 - bottom**3) / radius)
    return {"potential": potential, "g_z": 1e5 * potential / radius}


def variable_shell(bottom, top, shape=(6, 12)):
    n_lat, n_lon = shape
    longitude = np.linspace(-180, 180, n_lon + 1)
    latitude = np.linspace(-90, 90, n_lat + 1)
    return np.array([[w, e, s, n, bottom, top]
                     for w, e in zip(longitude[:-1], longitude[1:], strict=True)
                     for s, n in zip(latitude[:-1], latitude[1:], strict=True)])


def shell_surface_points(top):
    lon, lat = np.meshgrid(np.linspace(-180, 180, 13), np.linspace(-90, 90, 19))
    return (lon, lat, np.full(lon.shape, top))


@pytest.mark.parametrize("field", ["potential", "g_z"])
@pytest.mark.parametrize("thickness", [1e2, 1e3, 1e6])
def test_oracle_shell_linear_density(field, thickness):
    """test/test_tesseroid_variable_density.py:441-479 on the oracle."""
    top = 6371e3
    bottom = top - thickness
    slope = (2500.0 - 3300.0) / (top - bottom)
    constant = 2500.0 - slope * top
    fn = linear_shell_density(top, bottom)
    tess = ht.density_based_discretization(variable_shell(bottom, top), fn)
    coords = shell_surface_points(top)
    got = to.tesseroid_gravity(coords, tess, None, field, node_density=node_densities(tess, fn))
    npt.assert_allclose(got, analytic_shell_linear(top, bottom, top, slope, constant)[field],
                        rtol=ACCURACY_THRESHOLD)


@pytest.mark.parametrize("field", ["potential", "g_z"])
@pytest.mark.parametrize("thickness", [1e2, 1e3, 1e6])
@pytest.mark.parametrize("b_factor", [5, 100])
def test_oracle_shell_exponential_density(field, thickness, b_factor):
    """test/test_tesseroid_variable_density.py:482-525 on the oracle."""
    top = 6371e3
    bottom = top - thickness
    a_factor = (3300.0 - 2670.0) / (1 - np.exp(-b_factor))
    constant = 3300.0 - a_factor
    fn = exponential_shell_density(top, bottom, b_factor)
    tess = ht.density_based_discretization(variable_shell(bottom, top), fn)
    coords = shell_surface_points(top)
    got = to.tesseroid_gravity(coords, tess, None, field, node_density=node_densities(tess, fn))
    expected = analytic_shell_exponential(top, bottom, top, a_factor, b_factor, constant)[field]
    npt.assert_allclose(got, expected, rtol=ACCURACY_THRESHOLD)
