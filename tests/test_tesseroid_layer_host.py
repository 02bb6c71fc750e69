"""
Tesseroid layer container and accessor on the CPU (construction, checks,
boundaries, NaN masks, thin-tesseroid discard), mirroring
test/test_tesseroid_layer.py of the reference.  The gravity of the layer is
tested on the GPU in test_gpu_tesseroid_layer.py.
"""

import warnings

import numpy as np
import numpy.testing as npt
import pytest

from harmonica_gb300.tesseroid_layer import _discard_thin_tesseroids, tesseroid_layer

MEAN_RADIUS = 6371008.8


@pytest.fixture(params=("numpy", "reference-as-array"))
def dummy_layer(request):
    latitude = np.linspace(-10, 10, 6)
    longitude = np.linspace(-10, 10, 5)
    shape = (latitude.size, longitude.size)
    surface = MEAN_RADIUS * np.ones(shape) + 1e3
    reference = MEAN_RADIUS
    if request.param == "reference-as-array":
        reference *= np.ones(shape)
    density = 2670 * np.ones(shape)
    return (longitude, latitude), surface, reference, density


@pytest.mark.parametrize(("west", "east"), [(0, 480), (0, 360), (-180, 180), (0, 360 - 18 / 2)])
def test_overlap_invalid(west, east):
    latitude = np.linspace(-10, 10, 6)
    longitude = np.linspace(west, east, 21)
    shape = (latitude.size, longitude.size)
    msg = ("Found invalid longitude coordinates that would create "
           "overlapping tesseroids around the globe.")
    with pytest.raises(ValueError, match=msg):
        tesseroid_layer((longitude, latitude), MEAN_RADIUS * np.ones(shape) + 1e3,
                        MEAN_RADIUS * np.ones(shape))


@pytest.mark.parametrize(("west", "east"), [(0, 360 - 18), (-180, 180 - 18)])
def test_overlap_valid(west, east):
    latitude = np.linspace(-10, 10, 6)
    longitude = np.linspace(west, east, 21)
    shape = (latitude.size, longitude.size)
    tesseroid_layer((longitude, latitude), MEAN_RADIUS * np.ones(shape) + 1e3,
                    MEAN_RADIUS * np.ones(shape))


def test_layer_top_bottom(dummy_layer):
    (longitude, latitude), surface, reference, _ = dummy_layer
    layer = tesseroid_layer((longitude, latitude), surface, reference)
    for name in ("latitude", "longitude", "top", "bottom"):
        assert name in layer.coords
    npt.assert_allclose(layer.latitude, latitude)
    npt.assert_allclose(layer.longitude, longitude)
    npt.assert_allclose(layer.top, surface)
    npt.assert_allclose(layer.bottom, reference * np.ones(surface.shape))
    surface = surface.copy()
    surface[1, 1] = MEAN_RADIUS - 1e3
    layer = tesseroid_layer((longitude, latitude), surface, reference)
    assert layer.top[1, 1] == MEAN_RADIUS and layer.bottom[1, 1] == MEAN_RADIUS - 1e3


def test_invalid_surface_reference(dummy_layer):
    coords, surface, reference, _ = dummy_layer
    with pytest.raises(ValueError, match="Invalid surface array with shape"):
        tesseroid_layer(coords, np.arange(20, dtype=float), reference)
    with pytest.raises(ValueError, match="Invalid reference array with shape"):
        tesseroid_layer(coords, surface, np.zeros(20))


def test_properties(dummy_layer):
    coords, surface, reference, density = dummy_layer
    layer = tesseroid_layer(coords, surface, reference,
                            properties={"density": density, "suceptibility": 0 * density + 1e-3})
    npt.assert_allclose(layer.density, density)
    npt.assert_allclose(layer.suceptibility, 1e-3)


def test_no_regular_grid(dummy_layer):
    (longitude, latitude), surface, reference, _ = dummy_layer
    bad = longitude.copy()
    bad[3] = -22
    with pytest.raises(ValueError, match="Passed longitude coordinates are not evenly spaced."):
        tesseroid_layer((bad, latitude), surface, reference)
    bad = latitude.copy()
    bad[3] = -22
    with pytest.raises(ValueError, match="Passed latitude coordinates are not evenly spaced."):
        tesseroid_layer((longitude, bad), surface, reference)


def test_attributes():
    latitude = np.linspace(-10, 10, 6)
    longitude = np.linspace(-10, 10, 5)
    shape = (latitude.size, longitude.size)
    surface = MEAN_RADIUS * np.ones(shape)
    layer = tesseroid_layer((longitude, latitude), surface, surface - 1e3)
    acc = layer.tesseroid_layer
    assert acc.dims == ("latitude", "longitude")
    assert acc.spacing == (4, 5)
    assert acc.boundaries == (longitude[0] - 2.5, longitude[-1] + 2.5, latitude[0] - 2,
                              latitude[-1] + 2)
    assert acc.size == 30 and acc.shape == (6, 5)
    assert layer.attrs["radius_units"] == "meters"


def test_to_tesseroids_and_get_tesseroid():
    latitude = np.linspace(-1, 1, 2)
    longitude = np.linspace(-2, 2, 2)
    surface = MEAN_RADIUS * np.ones((2, 2))
    layer = tesseroid_layer((longitude, latitude), surface, surface - 1e3)
    b, t = MEAN_RADIUS - 1e3, MEAN_RADIUS
    expected = [[-4.0, 0.0, -2.0, 0.0, b, t], [0.0, 4.0, -2.0, 0.0, b, t],
                [-4.0, 0.0, 0.0, 2.0, b, t], [0.0, 4.0, 0.0, 2.0, b, t]]
    npt.assert_allclose(layer.tesseroid_layer._to_tesseroids(), expected)
    for i in range(2):
        for j in range(2):
            npt.assert_allclose(layer.tesseroid_layer.get_tesseroid((i, j)), expected[2 * i + j])


def test_nonans_mask(dummy_layer):
    (longitude, latitude), surface, reference, _ = dummy_layer
    shape = (latitude.size, longitude.size)
    layer = tesseroid_layer((longitude, latitude), surface, reference)
    npt.assert_array_equal(layer.tesseroid_layer._get_nonans_mask(), np.ones(shape, bool))
    expected = np.ones(shape, bool)
    for index in ((1, 2), (2, 3)):
        layer.top[index] = np.nan
        expected[index] = False
    for index in ((1, 2), (2, 1), (3, 2)):
        layer.bottom[index] = np.nan
        expected[index] = False
    npt.assert_array_equal(layer.tesseroid_layer._get_nonans_mask(), expected)


def test_nonans_mask_property_warning(dummy_layer):
    coords, surface, reference, density = dummy_layer
    shape = surface.shape
    surface, density = surface.copy(), density.copy()
    expected = np.ones(shape, bool)
    for index in ((1, 2), (2, 3)):
        surface[index] = np.nan
        density[index] = np.nan
        expected[index] = False
    layer = tesseroid_layer(coords, surface, reference, properties={"density": density})
    with warnings.catch_warnings(record=True) as warn:
        warnings.simplefilter("always")
        mask = layer.tesseroid_layer._get_nonans_mask(property_name="density")
        assert len(warn) == 0
    npt.assert_array_equal(mask, expected)
    density = 2670 * np.ones(shape)
    for index in ((2, 2), (0, 1)):
        density[index] = np.nan
        expected[index] = False
    layer = tesseroid_layer(coords, surface, reference, properties={"density": density})
    with warnings.catch_warnings(record=True) as warn:
        warnings.simplefilter("always")
        mask = layer.tesseroid_layer._get_nonans_mask(property_name="density")
        assert len(warn) == 1 and issubclass(warn[-1].category, UserWarning)
        assert "Found missing values in 'density' property" in str(warn[-1].message)
    npt.assert_array_equal(mask, expected)


def test_discard_thin_tesseroids():
    """test/test_tesseroid_layer.py:535-560."""
    tess = np.array([[-5, 5, -5, 5, MEAN_RADIUS - 1e3, MEAN_RADIUS],
                     [-5, 5, -5, 5, MEAN_RADIUS - 1, MEAN_RADIUS],
                     [-5, 5, -5, 5, MEAN_RADIUS - 1e-2, MEAN_RADIUS],
                     [-5, 5, -5, 5, MEAN_RADIUS - 1e2, MEAN_RADIUS]])
    dens = np.array([2670.0, 2000.0, 1900.0, 3000.0])
    t, d = _discard_thin_tesseroids(tess, dens, 10)
    npt.assert_allclose(t, tess[[0, 3]])
    npt.assert_allclose(d, [2670.0, 3000.0])
