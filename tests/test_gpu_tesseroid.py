"""
Tesseroid forward model on the GPU (hg_tesseroid_forward, hg_tesseroid_inside
through harmonica_gb300.tesseroid_gravity) against harmonica's own outputs,
the oracle and the analytic spherical shell; the checks and errors of
test/test_tesseroid.py.

Tolerances.  The kernel follows the reference's operation order without
fused multiply-adds, so it differs from the reference (and the oracle) only
through the last bits of CUDA's cos/sin/acos.  How far that moves a result is
a property of the reference's algorithm, measured on the CPU by
test_tesseroid_host.py::test_oracle_libm_sensitivity (every cos/sin/acos
nudged by one ulp): points far above the model move by ~1e-13, points a
kilometre or less from a tesseroid by up to ~1e-9 (cancellation in
1 - cos(psi) of the distance formula), and points ON a tesseroid face by up
to 8e-4 on a 10 m shell: there the reference splits small tesseroids many
levels deep and its size formula (top * arccos(...), _tesseroid_utils.py:
274-279) loses half its digits, so one distance / size < ratio decision can
flip.  Hence rtol 1e-11 far, 1e-8 near and 1e-3 (the reference's own
ACCURACY_THRESHOLD) on faces.
"""

import re

import numpy as np
import numpy.testing as npt
import pytest

torch = pytest.importorskip("torch")

import harmonica_gb300 as hg  # noqa: E402
from harmonica_gb300 import tesseroid as ht  # noqa: E402
from oracle import tesseroid_oracle as to  # noqa: E402

from test_tesseroid_host import (  # noqa: E402
    ACCURACY_THRESHOLD,
    MEAN_RADIUS,
    _var_golden,
    analytic_shell_exponential,
    analytic_shell_linear,
    exponential_shell_density,
    golden_case,
    golden_keys,
    linear_shell_density,
    shell,
    shell_surface_points,
    variable_density_fn,
    variable_keys,
    variable_shell,
)

pytestmark = pytest.mark.gpu

NEAR_RTOL = 1e-8
FAR_RTOL = 1e-11
SURFACE_RTOL = ACCURACY_THRESHOLD
# golden cases whose points lie on a tesseroid face
ON_SURFACE = ("shell2d_surface", "disable_checks")


@pytest.mark.parametrize("key", golden_keys())
def test_gpu_matches_reference(key):
    coords, tess, dens, field, radial, disable, expected = golden_case(key)
    got = hg.tesseroid_gravity(coords, tess, dens, field, radial_adaptive_discretization=radial,
                               disable_checks=disable)
    scale = np.max(np.abs(expected))
    rtol = SURFACE_RTOL if key.startswith(ON_SURFACE) else NEAR_RTOL
    npt.assert_allclose(got.ravel(), expected, rtol=rtol, atol=1e-15 * scale)


def random_model(seed, n_tess, n_points, min_height, max_height):
    rng = np.random.default_rng(seed)
    w = rng.uniform(-30, 25, n_tess)
    s = rng.uniform(-30, 25, n_tess)
    top = MEAN_RADIUS - rng.uniform(0, 3e3, n_tess)
    tess = np.stack([w, w + rng.uniform(0.2, 5, n_tess), s, s + rng.uniform(0.2, 5, n_tess),
                     top - rng.uniform(500, 50e3, n_tess), top], axis=1)
    dens = rng.uniform(-600, 3300, n_tess)
    coords = (rng.uniform(-35, 35, n_points), rng.uniform(-35, 35, n_points),
              MEAN_RADIUS + rng.uniform(min_height, max_height, n_points))
    return coords, tess, dens


@pytest.mark.parametrize("field", ["potential", "g_z"])
@pytest.mark.parametrize("radial", [False, True])
def test_gpu_random_model_vs_oracle(field, radial):
    coords, tess, dens = random_model(11, 300, 500, 100.0, 80e3)
    got = hg.tesseroid_gravity(coords, tess, dens, field, radial_adaptive_discretization=radial)
    ref = to.tesseroid_gravity(coords, tess, dens, field, radial_adaptive_discretization=radial)
    npt.assert_allclose(got, ref, rtol=NEAR_RTOL, atol=1e-14 * np.max(np.abs(ref)))


@pytest.mark.parametrize("field", ["potential", "g_z"])
def test_gpu_far_points_vs_oracle(field):
    """Points 20-80 km above the model: last-bit agreement class."""
    coords, tess, dens = random_model(12, 300, 400, 20e3, 80e3)
    got = hg.tesseroid_gravity(coords, tess, dens, field)
    ref = to.tesseroid_gravity(coords, tess, dens, field)
    npt.assert_allclose(got, ref, rtol=FAR_RTOL, atol=1e-14 * np.max(np.abs(ref)))


@pytest.mark.parametrize("field", ["potential", "g_z"])
def test_gpu_dense_near_pairs(field):
    """Points 1-3 km above a 60 x 60 grid of 0.1-degree tesseroids: every warp
    queues hundreds of split pairs (several flushes of its list)."""
    lon = np.linspace(-3, 3, 61)
    lat = np.linspace(-3, 3, 61)
    tess = np.array([[w, e, s, n, MEAN_RADIUS - 2e3, MEAN_RADIUS]
                     for w, e in zip(lon[:-1], lon[1:], strict=True)
                     for s, n in zip(lat[:-1], lat[1:], strict=True)])
    rng = np.random.default_rng(5)
    dens = rng.uniform(2000, 3000, tess.shape[0])
    coords = (rng.uniform(-2.5, 2.5, 200), rng.uniform(-2.5, 2.5, 200),
              MEAN_RADIUS + rng.uniform(1e3, 3e3, 200))
    got = hg.tesseroid_gravity(coords, tess, dens, field)
    ref = to.tesseroid_gravity(coords, tess, dens, field)
    npt.assert_allclose(got, ref, rtol=NEAR_RTOL)


def test_gpu_many_chunks_and_determinism():
    """More tesseroids than one chunk (partials reduced in fixed order);
    repeated runs are bit-identical."""
    coords, tess, dens = random_model(3, 20000, 64, 1e3, 30e3)
    a = hg.tesseroid_gravity(coords, tess, dens, "g_z")
    b = hg.tesseroid_gravity(coords, tess, dens, "g_z")
    npt.assert_array_equal(a, b)
    ref = to.tesseroid_gravity(coords, tess, dens, "g_z")
    npt.assert_allclose(a, ref, rtol=NEAR_RTOL)


@pytest.mark.parametrize("field", ["potential", "g_z"])
@pytest.mark.parametrize("thickness", [10, 100, 1e3, 1e4, 1e5])
def test_gpu_spherical_shell_3d(field, thickness):
    """test/test_tesseroid.py:729-770."""
    radius = MEAN_RADIUS + 1e3
    top, bottom = MEAN_RADIUS, MEAN_RADIUS - thickness
    got = hg.tesseroid_gravity([0, 0, radius], shell((6, 6), bottom, top), np.full(36, 1000.0),
                               field, radial_adaptive_discretization=True)
    npt.assert_allclose(got, to.spherical_shell(top, bottom, 1000, radius)[field],
                        rtol=ACCURACY_THRESHOLD)


@pytest.mark.parametrize("field", ["potential", "g_z"])
def test_gpu_spherical_shell_2d(field):
    """test/test_tesseroid.py:683-726 (points on the top surface)."""
    lon, lat = np.meshgrid(np.arange(0, 351, 10.0), np.arange(-90, 91, 10.0))
    coords = (lon, lat, np.full(lon.shape, MEAN_RADIUS))
    for thickness in np.logspace(1, 5, 5):
        tess = shell((12, 6), MEAN_RADIUS - thickness, MEAN_RADIUS)
        got = hg.tesseroid_gravity(coords, tess, np.full(72, 1000.0), field)
        expected = to.spherical_shell(MEAN_RADIUS, MEAN_RADIUS - thickness, 1000,
                                      MEAN_RADIUS)[field]
        npt.assert_allclose(got, expected, rtol=ACCURACY_THRESHOLD)
        npt.assert_allclose(got, to.tesseroid_gravity(coords, tess, np.full(72, 1000.0), field),
                            rtol=SURFACE_RTOL)


@pytest.mark.parametrize("field", ["potential", "g_z"])
def test_gpu_longitude_continuity_equivalent(field):
    """test/test_tesseroid.py:444-462."""
    top, bottom = MEAN_RADIUS, MEAN_RADIUS - 1e4
    coords = [0, 0, MEAN_RADIUS + 1e3]
    a = hg.tesseroid_gravity(coords, [-10, 10, -10, 10, bottom, top], 1e3, field=field)
    b = hg.tesseroid_gravity(coords, [350, 10, -10, 10, bottom, top], 1e3, field=field)
    npt.assert_allclose(a, b)


def test_gpu_disable_checks():
    """test/test_tesseroid.py:224-244."""
    valid = [0.0, 10.0, 0.0, 10.0, 10.0, 20.0]
    invalid = [0.0, 10.0, 0.0, 10.0, 20.0, 10.0]
    coords = [0.0, 0.0, 10.0]
    with pytest.raises(ValueError, match="The bottom radius boundary can't be greater"):
        hg.tesseroid_gravity(coords, invalid, 100.0, field="potential")
    bad = hg.tesseroid_gravity(coords, invalid, 100.0, field="potential", disable_checks=True)
    good = hg.tesseroid_gravity(coords, valid, 100.0, field="potential")
    npt.assert_allclose(bad, -good)


def test_gpu_invalid_density_array():
    """test/test_tesseroid.py:112-131."""
    tess = [[-10, 0, -10, 0, 100, 200], [-10, 0, 0, 10, 100, 200],
            [0, 10, -10, 0, 100, 200], [0, 10, 0, 10, 100, 200]]
    msg = r"Number of elements in density \([0-9]+\) mismatch the number of tesseroids \([0-9]+\)"
    with pytest.raises(ValueError, match=msg):
        hg.tesseroid_gravity([0, 0, 250], tess, [1000, 2000], field="potential")


def test_gpu_variable_density_radial_not_supported():
    with pytest.raises(NotImplementedError, match="radial_adaptive_discretization"):
        hg.tesseroid_gravity([0, 0, 250], [-10, 10, -10, 10, 100, 200], lambda r: 1.0,
                             field="potential", radial_adaptive_discretization=True)


@pytest.mark.parametrize("key", variable_keys())
def test_gpu_variable_density_matches_reference(key):
    """Density functions (density-based discretization on the host, density
    per radial node on the GPU) against harmonica's own results; points on
    the shell's top face take the on-face tolerance."""
    g = _var_golden()
    name = key.rsplit("_", 2)[0] if key.endswith("g_z") else key.rsplit("_", 1)[0]
    field = "g_z" if key.endswith("g_z") else "potential"
    coords = tuple(g[f"{key}_coords"])
    tess = g[f"{key}_tesseroids"]
    got = hg.tesseroid_gravity(coords, tess, variable_density_fn(name), field=field).ravel()
    expected = g[f"{key}_result"]
    on_face = np.isin(coords[2], tess[:, 5])
    npt.assert_allclose(got[~on_face], expected[~on_face], rtol=NEAR_RTOL)
    npt.assert_allclose(got[on_face], expected[on_face], rtol=SURFACE_RTOL)


@pytest.mark.parametrize("field", ["potential", "g_z"])
def test_gpu_single_tesseroid_against_constant_density(field):
    """test/test_tesseroid_variable_density.py:321-355."""
    bottom, top = 5400e3, 6300e3
    tess = [-3, 3, -2, 2, bottom, top]
    lon, lat = np.meshgrid(np.arange(-5, 5.1, 1.0), np.arange(-5, 5.1, 1.0))
    coords = (lon, lat, np.full(lon.shape, top))
    npt.assert_allclose(hg.tesseroid_gravity(coords, [tess], [2900.0], field=field),
                        hg.tesseroid_gravity(coords, [tess], lambda r: 2900.0, field=field))


@pytest.mark.parametrize("field", ["potential", "g_z"])
@pytest.mark.parametrize("thickness", [1e2, 1e3, 1e6])
def test_gpu_shell_linear_density(field, thickness):
    """test/test_tesseroid_variable_density.py:441-479."""
    top = 6371e3
    bottom = top - thickness
    slope = (2500.0 - 3300.0) / (top - bottom)
    constant = 2500.0 - slope * top
    got = hg.tesseroid_gravity(shell_surface_points(top), variable_shell(bottom, top),
                               linear_shell_density(top, bottom), field=field)
    npt.assert_allclose(got, analytic_shell_linear(top, bottom, top, slope, constant)[field],
                        rtol=ACCURACY_THRESHOLD)


@pytest.mark.parametrize("field", ["potential", "g_z"])
@pytest.mark.parametrize("thickness", [1e2, 1e3, 1e6])
@pytest.mark.parametrize("b_factor", [5, 100])
def test_gpu_shell_exponential_density(field, thickness, b_factor):
    """test/test_tesseroid_variable_density.py:482-525."""
    top = 6371e3
    bottom = top - thickness
    a_factor = (3300.0 - 2670.0) / (1 - np.exp(-b_factor))
    constant = 3300.0 - a_factor
    got = hg.tesseroid_gravity(shell_surface_points(top), variable_shell(bottom, top),
                               exponential_shell_density(top, bottom, b_factor), field=field)
    expected = analytic_shell_exponential(top, bottom, top, a_factor, b_factor, constant)[field]
    npt.assert_allclose(got, expected, rtol=ACCURACY_THRESHOLD)


INSIDE = re.escape("Found computation point(s) inside tesseroid(s)")


def test_gpu_points_outside_pass():
    """test/test_tesseroid.py:251-267: points on faces are outside."""
    points = np.array([[0, 0, 250], [20, 0, 150], [0, 20, 150], [0, 0, 200], [0, 0, 100],
                       [-10, 0, 150], [10, 0, 150], [0, -10, 150], [0, 10, 150]], float).T
    ht.check_points_outside_tesseroids(points, np.atleast_2d([-10, 10, -10, 10, 100, 200.0]))


@pytest.mark.parametrize("point", [[0, 0, 150], [360, 0, 150]])
def test_gpu_point_inside(point):
    """test/test_tesseroid.py:270-277."""
    with pytest.raises(ValueError, match=INSIDE):
        ht.check_points_outside_tesseroids(np.atleast_2d(np.array(point, float)).T,
                                           np.atleast_2d([-10, 10, -10, 10, 100, 200.0]))


@pytest.mark.parametrize(("point", "tess"), [([360, 0, 150], [-10, 10, -10, 10, 100, 200]),
                                             ([-90, 0, 150], [260, 280, -10, 10, 100, 200])])
def test_gpu_point_phased_longitude(point, tess):
    """test/test_tesseroid.py:280-293."""
    with pytest.raises(ValueError, match=INSIDE):
        ht.check_points_outside_tesseroids(np.atleast_2d(np.array(point, float)).T,
                                           np.atleast_2d(np.array(tess, float)))


def test_gpu_multiple_points_inside_message():
    """test/test_tesseroid.py:296-315, with the full message: every
    conflicting pair, point-major order."""
    tess = np.array([[-10, 10, -10, 10, 100, 200], [20, 30, 20, 30, 400, 500],
                     [-50, -40, -30, -20, 100, 500]], float)
    points = np.array([[0, 0, 150], [80, 82, 4000], [10, 10, 450], [25, 25, 450]], float).T
    with pytest.raises(ValueError, match=INSIDE) as err:
        hg.tesseroid_gravity(tuple(points), tess, [1.0, 1.0, 1.0], field="potential")
    msg = str(err.value)
    assert msg.count(" - Computation point") == 2
    first = msg.index("'(0.0, 0.0, 150.0)' inside tesseroid '(-10.0, 10.0, -10.0, 10.0, 100.0")
    second = msg.index("'(25.0, 25.0, 450.0)' inside tesseroid '(20.0, 30.0, 20.0, 30.0, 400.0")
    assert first < second


def test_gpu_stack_overflow_through_api():
    """A point on the top face with the radial split overflows the stack of
    100 (the oracle agrees)."""
    tess = [[-1, 1, -1, 1, MEAN_RADIUS - 1e3, MEAN_RADIUS]]
    with pytest.raises(OverflowError, match="Stack Overflow"):
        to.tesseroid_gravity([0, 0, MEAN_RADIUS], tess, [1000.0], "g_z",
                             radial_adaptive_discretization=True)
    with pytest.raises(OverflowError, match="Stack Overflow"):
        hg.tesseroid_gravity([0, 0, MEAN_RADIUS], tess, [1000.0], "g_z",
                             radial_adaptive_discretization=True)


def test_gpu_overflow_limits(monkeypatch):
    """test/test_tesseroid.py:318-336 through the module constants: a stack
    of 2 and at most 2 small tesseroids."""
    coords = [0.0, 0.0, MEAN_RADIUS + 10.0]
    tess = [-10.0, 10.0, -10.0, 10.0, MEAN_RADIUS - 1e3, MEAN_RADIUS]
    monkeypatch.setattr(ht, "STACK_SIZE", 2)
    with pytest.raises(OverflowError, match="Stack Overflow"):
        hg.tesseroid_gravity(coords, tess, 1000.0, field="g_z")
    monkeypatch.setattr(ht, "STACK_SIZE", 100)
    monkeypatch.setattr(ht, "MAX_DISCRETIZATIONS", 2)
    with pytest.raises(OverflowError, match="Exceeded maximum discretizations"):
        hg.tesseroid_gravity(coords, tess, 1000.0, field="g_z")


def test_gpu_null_tesseroids_skipped():
    """Zero-volume and zero-density tesseroids contribute nothing
    (_discard_null_tesseroids), even next to the points."""
    coords, tess, dens = random_model(7, 50, 40, 500.0, 20e3)
    extra = tess[:6].copy()
    extra[0, 1] = extra[0, 0]
    extra[1, 3] = extra[1, 2]
    extra[2, 4] = extra[2, 5]
    extra_dens = np.array([1e3, 1e3, 1e3, 0.0, 0.0, 0.0])
    a = hg.tesseroid_gravity(coords, tess, dens, "g_z")
    b = hg.tesseroid_gravity(coords, np.vstack([extra, tess]), np.concatenate([extra_dens, dens]),
                             "g_z")
    npt.assert_allclose(a, b, rtol=1e-13)


def test_gpu_shapes_and_dtype():
    lon, lat = np.meshgrid(np.linspace(-5, 5, 7), np.linspace(-4, 4, 5))
    coords = (lon, lat, np.full(lon.shape, MEAN_RADIUS + 5e3))
    tess = [[-1, 1, -1, 1, MEAN_RADIUS - 1e4, MEAN_RADIUS]]
    out = hg.tesseroid_gravity(coords, tess, [2670.0], "g_z", dtype=np.float32)
    assert out.shape == lon.shape and out.dtype == np.float32
    ref = to.tesseroid_gravity(coords, tess, [2670.0], "g_z")
    npt.assert_allclose(out, ref.astype(np.float32), rtol=1e-6)
    single = hg.tesseroid_gravity([0.0, 0.0, MEAN_RADIUS + 1e3], tess, 2670.0, "potential")
    assert np.ndim(single) == 0 or single.shape == ()


@pytest.mark.parametrize("field", ["potential", "g_z"])
def test_gpu_parallel_and_progressbar_flags(field):
    """test/test_tesseroid.py (parallel and progress-bar tests): results with
    parallel=False and with the progress bar equal the defaults."""
    coords, tess, dens = random_model(12, 40, 60, 100.0, 50e3)
    base = hg.tesseroid_gravity(coords, tess, dens, field)
    npt.assert_array_equal(hg.tesseroid_gravity(coords, tess, dens, field, parallel=False), base)
    npt.assert_array_equal(hg.tesseroid_gravity(coords, tess, dens, field, progressbar=True),
                           base)
