"""
Gravity of a tesseroid layer on the GPU (harmonica_gb300.tesseroid_layer
accessor), mirroring test/test_tesseroid_layer.py:387-533 of the reference:
the layer's field equals tesseroid_gravity of its tesseroids, NaN tops and
densities drop their tesseroids (with the reference's warning), thin
tesseroids are discarded.
"""

import warnings

import numpy as np
import numpy.testing as npt
import pytest

pytest.importorskip("torch")

import harmonica_gb300 as hg  # noqa: E402
from harmonica_gb300.tesseroid_layer import tesseroid_layer  # noqa: E402
from oracle import tesseroid_oracle as to  # noqa: E402

pytestmark = pytest.mark.gpu

MEAN_RADIUS = 6371008.8


def dummy():
    latitude = np.linspace(-10, 10, 6)
    longitude = np.linspace(-10, 10, 5)
    shape = (latitude.size, longitude.size)
    surface = MEAN_RADIUS * np.ones(shape) + 1e3
    density = 2670 * np.ones(shape)
    lon, lat = np.meshgrid(np.arange(-10, 10.1, 7.0), np.arange(-10, 10.1, 7.0))
    grid = (lon, lat, np.full(lon.shape, surface[0, 0] + 10e3))
    return (longitude, latitude), surface, MEAN_RADIUS, density, grid


def holes(layer, density, indices):
    tess = [layer.tesseroid_layer.get_tesseroid((i, j)) for i in range(6) for j in range(5)
            if (i, j) not in indices]
    rho = [density[i, j] for i in range(6) for j in range(5) if (i, j) not in indices]
    return np.array(tess, dtype=float), np.array(rho, dtype=float)


@pytest.mark.parametrize("field", ["potential", "g_z"])
def test_layer_gravity(field):
    coords, surface, reference, density, grid = dummy()
    layer = tesseroid_layer(coords, surface, reference, properties={"density": density})
    expected = hg.tesseroid_gravity(grid, layer.tesseroid_layer._to_tesseroids(),
                                    density.ravel(), field=field)
    npt.assert_allclose(layer.tesseroid_layer.gravity(grid, field=field), expected)
    ref = to.tesseroid_gravity(grid, layer.tesseroid_layer._to_tesseroids(), density.ravel(),
                               field)
    # points 10 km above 4-5 degree tesseroids that are split: the near class
    # of test_gpu_tesseroid.py
    npt.assert_allclose(expected, ref, rtol=1e-8)


@pytest.mark.parametrize("field", ["potential", "g_z"])
def test_layer_gravity_surface_nans(field):
    coords, surface, reference, density, grid = dummy()
    indices = [(3, 3), (2, 1)]
    full = tesseroid_layer(coords, surface, reference, properties={"density": density})
    tess, rho = holes(full, density, indices)
    surface = surface.copy()
    for index in indices:
        surface[index] = np.nan
    layer = tesseroid_layer(coords, surface, reference, properties={"density": density})
    npt.assert_allclose(layer.tesseroid_layer.gravity(grid, field=field),
                        hg.tesseroid_gravity(grid, tess, rho, field=field))


@pytest.mark.parametrize("field", ["potential", "g_z"])
def test_layer_gravity_density_nans(field):
    coords, surface, reference, density, grid = dummy()
    indices = [(3, 3), (2, 1)]
    full = tesseroid_layer(coords, surface, reference, properties={"density": density})
    tess, rho = holes(full, density, indices)
    density = density.copy()
    for index in indices:
        density[index] = np.nan
    layer = tesseroid_layer(coords, surface, reference, properties={"density": density})
    with warnings.catch_warnings(record=True) as warn:
        warnings.simplefilter("always")
        result = layer.tesseroid_layer.gravity(grid, field=field)
        assert len(warn) == 1
    npt.assert_allclose(result, hg.tesseroid_gravity(grid, tess, rho, field=field))


def test_layer_gravity_discards_thin_tesseroids():
    """test/test_tesseroid_layer.py:495-533."""
    coords, surface, reference, density, grid = dummy()
    surface = surface.copy()
    surface[3, 3] = MEAN_RADIUS + 1e-3
    surface[2, 1] = MEAN_RADIUS + 1e-2
    layer = tesseroid_layer(coords, surface, reference, properties={"density": density})
    tess, rho = holes(layer, density, [(3, 3), (2, 1)])
    npt.assert_allclose(layer.tesseroid_layer.gravity(grid, field="g_z", thickness_threshold=1),
                        hg.tesseroid_gravity(grid, tess, rho, field="g_z"))


def test_layer_progress_bar():
    """test/test_tesseroid_layer.py (progress-bar test): the accessor's
    results with and without the progress bar match."""
    coords, surface, reference, density, grid = dummy()
    layer = tesseroid_layer(coords, surface, reference, properties={"density": density})
    npt.assert_allclose(layer.tesseroid_layer.gravity(grid, field="g_z", progressbar=True),
                        layer.tesseroid_layer.gravity(grid, field="g_z", progressbar=False))
