"""
Property-based tests (hypothesis) of host helpers: shard partitions, chunk
sizes of the serving loop, longitude continuity of tesseroids, the prism
boundary check and the magnetic vector conversions.  CPU only; skipped where
hypothesis is not installed.
"""

import numpy as np
import numpy.testing as npt
import pytest

try:
    import hypothesis
    import hypothesis.strategies as st
except ImportError:  # the GPU image has no hypothesis: these CPU tests are skipped there
    hypothesis = None

    class _Anything:
        """Stands in for hypothesis' strategies and decorators when it is
        absent, so that the module still imports (and its tests skip)."""

        def __getattr__(self, name):
            return self

        def __call__(self, *args, **kwargs):
            return args[0] if len(args) == 1 and callable(args[0]) and not kwargs else self

    st = _Anything()
    given = settings = _Anything()
else:
    given, settings = hypothesis.given, hypothesis.settings

pytestmark = pytest.mark.skipif(hypothesis is None, reason="hypothesis is not installed")

from harmonica_gb300.gravity import check_prisms  # noqa: E402
from harmonica_gb300.magnetic_utils import (  # noqa: E402
    magnetic_angles_to_vec,
    magnetic_vec_to_angles,
)
from harmonica_gb300.serve import chunk_for  # noqa: E402
from harmonica_gb300.sharding import shard_bounds  # noqa: E402
from harmonica_gb300.tesseroid import longitude_continuity  # noqa: E402

FAST = settings(max_examples=200, deadline=None)


@FAST
@given(st.integers(0, 10**7), st.integers(1, 64))
def test_shards_partition_the_points(n, world):
    spans = [shard_bounds(n, r, world) for r in range(world)]
    assert spans[0][0] == 0 and spans[-1][1] == n
    assert all(a[1] == b[0] for a, b in zip(spans, spans[1:]))
    sizes = [hi - lo for lo, hi in spans]
    assert min(sizes) >= 0 and max(sizes) - min(sizes) <= 1


@FAST
@given(st.integers(0, 10**8), st.integers(128, 1 << 16))
def test_chunks_are_whole_tiles(n_prisms, max_chunk):
    chunk = chunk_for(n_prisms, max_chunk)
    assert chunk % 128 == 0 and 128 <= chunk <= max(128, max_chunk)
    if n_prisms <= (max_chunk // 128) * 128:
        assert chunk >= n_prisms  # one chunk holds the whole request


_lon = st.floats(-180, 360, allow_nan=False)


@FAST
@given(st.lists(st.tuples(_lon, _lon), min_size=1, max_size=20))
def test_longitude_continuity(pairs):
    tess = np.array([[w, e, -1.0, 1.0, 1.0, 2.0] for w, e in pairs])
    out = longitude_continuity(tess)
    moved = tess[:, 0] > tess[:, 1]
    # rows with west <= east are untouched, the others moved into [-180, 180)
    npt.assert_array_equal(out[~moved], tess[~moved])
    for col in (0, 1):
        new = out[moved, col]
        assert np.all((new >= -180) & (new < 180))
        # the same meridian: a whole number of turns apart
        turns = (tess[moved, col] - new) / 360.0
        npt.assert_allclose(turns, np.round(turns), atol=1e-9)
    npt.assert_array_equal(out[:, 2:], tess[:, 2:])


_coord = st.floats(-1e4, 1e4, allow_nan=False)


@FAST
@given(st.lists(st.tuples(*[_coord] * 6), min_size=1, max_size=10))
def test_check_prisms_raises_exactly_on_inverted_boundaries(rows):
    prisms = np.array(rows)
    bad = ((prisms[:, 0] > prisms[:, 1]) | (prisms[:, 2] > prisms[:, 3])
           | (prisms[:, 4] > prisms[:, 5]))
    if bad.any():
        with pytest.raises(ValueError, match="Invalid prism or prisms"):
            check_prisms(prisms)
    else:
        check_prisms(prisms)


@FAST
@given(st.floats(1e-3, 1e5), st.floats(-89.9, 89.9), st.floats(-179.9, 179.9))
def test_magnetic_angles_round_trip(intensity, inclination, declination):
    vec = magnetic_angles_to_vec(intensity, inclination, declination)
    npt.assert_allclose(magnetic_vec_to_angles(*vec), (intensity, inclination, declination),
                        rtol=1e-9, atol=1e-9)
    npt.assert_allclose(np.linalg.norm(vec), intensity, rtol=1e-12)


def _tesseroid_errors(t):
    """Whether the reference's checks reject these tesseroids (its order of
    conditions, longitudes made continuous before the west/east checks)."""
    w, e, s, n, b, top = (t[:, i].copy() for i in range(6))
    if np.any((s < -90) | (s > 90) | (n < -90) | (n > 90)) or np.any(s > n):
        return True
    if np.any((b < 0) | (top < 0)) or np.any(b > top):
        return True
    if np.any((w < -180) | (w > 360) | (e < -180) | (e > 360)):
        return True
    flip = w > e
    w[flip] = ((w[flip] + 180) % 360) - 180
    e[flip] = ((e[flip] + 180) % 360) - 180
    return bool(np.any(w > e) or np.any(e - w > 360))


_lat = st.floats(-95, 95, allow_nan=False)
_rad = st.floats(-1.0, 1e4, allow_nan=False)
_lon_wide = st.floats(-185, 365, allow_nan=False)


def _row(values):
    """Latitudes and radii put in order unless the flags leave them as drawn,
    so that valid and invalid tesseroids are both common."""
    w, e, s, n, b, t, keep_lat, keep_rad = values
    if not keep_lat:
        s, n = sorted((s, n))
    if not keep_rad:
        b, t = sorted((b, t))
    return [w, e, s, n, b, t]


@FAST
@given(st.lists(st.tuples(_lon_wide, _lon_wide, _lat, _lat, _rad, _rad,
                          st.booleans(), st.booleans()).map(_row),
                min_size=1, max_size=4))
def test_check_tesseroids_rejects_exactly_the_invalid(rows):
    from harmonica_gb300.tesseroid import check_tesseroids

    t = np.array(rows)
    if _tesseroid_errors(t):
        with pytest.raises(ValueError, match="Invalid tesseroid or tesseroids"):
            check_tesseroids(t)
    else:
        out = check_tesseroids(t)
        assert np.all(out[:, 0] <= out[:, 1])


@settings(max_examples=25, deadline=None)
@given(st.floats(-3.0, 3.0), st.floats(0.1, 5.0), st.floats(10.0, 5e3))
def test_density_based_discretization_tiles_the_radial_range(amplitude, rate, thickness):
    """The radial pieces of a tesseroid chain from its bottom to its top, in
    the reference's order of discovery, and keep its horizontal bounds."""
    from harmonica_gb300.tesseroid import density_based_discretization

    bottom, top = 6.3e6, 6.3e6 + thickness

    def density(radius):
        return 2670.0 + 300.0 * amplitude * np.exp(-rate * (radius - bottom) / thickness)

    pieces = density_based_discretization(np.array([[-1.0, 1.0, -2.0, 2.0, bottom, top]]),
                                          density)
    npt.assert_array_equal(pieces[:, :4], np.tile([-1.0, 1.0, -2.0, 2.0], (len(pieces), 1)))
    radial = pieces[np.argsort(pieces[:, 4]), 4:]
    assert radial[0, 0] == bottom and radial[-1, 1] == top
    npt.assert_array_equal(radial[1:, 0], radial[:-1, 1])
    assert np.all(radial[:, 0] < radial[:, 1])


@settings(max_examples=50, deadline=None)
@given(st.integers(2, 6), st.integers(2, 6), st.floats(1.0, 500.0), st.floats(1.0, 500.0),
       st.integers(0, 2**31 - 1))
def test_layer_prisms_index_and_order(n_north, n_east, s_north, s_east, seed):
    """prism_layer: top >= bottom with {top, bottom} = {surface, reference}
    on every cell, and ``get_prism((i, j))`` is row ``i * n_east + j`` of
    ``_to_prisms()`` (the reference's (northing, easting) order).  Two or
    more prisms per axis: like the reference, a one-prism axis has no
    spacing and fails the regular-grid check."""
    from harmonica_gb300 import prism_layer

    rng = np.random.default_rng(seed)
    easting = 1000.0 + s_east * np.arange(n_east)
    northing = -500.0 + s_north * np.arange(n_north)
    surface = rng.uniform(-1e3, 1e3, (n_north, n_east))
    reference = rng.uniform(-1e3, 1e3, (n_north, n_east))
    layer = prism_layer((easting, northing), surface, reference,
                        properties={"density": rng.uniform(2000, 3000, (n_north, n_east))})
    top, bottom = np.asarray(layer.top), np.asarray(layer.bottom)
    assert np.all(top >= bottom)
    npt.assert_array_equal(top, np.maximum(surface, reference))
    npt.assert_array_equal(bottom, np.minimum(surface, reference))
    prisms = layer.prism_layer._to_prisms()
    assert prisms.shape == (n_north * n_east, 6)
    for i in range(n_north):
        for j in range(n_east):
            npt.assert_array_equal(layer.prism_layer.get_prism((i, j)), prisms[i * n_east + j])
