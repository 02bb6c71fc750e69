"""
Host-side logic of the drop-in API (no GPU): argument errors, prism checks
and the prism-layer container, mirroring harmonica's test/test_prism.py and
test/test_prism_layer.py.
"""

import re

import numpy as np
import numpy.testing as npt
import pytest

import harmonica_gb300 as hg


def test_invalid_field():
    """test/test_prism.py:42-50"""
    msg = re.escape("Gravitational field this-field-does-not-exist not recognized")
    with pytest.raises(ValueError, match=msg):
        hg.prism_gravity([0, 0, 0], [-100, 100, -100, 100, -200, -100], 1000,
                         field="this-field-does-not-exist")


def test_invalid_density_array():
    """test/test_prism.py:53-70"""
    prisms = [
        [-100, 0, -100, 0, -200, -100],
        [-100, 0, 0, 100, -200, -100],
        [0, 100, -100, 0, -200, -100],
        [0, 100, 0, 100, -200, -100],
    ]
    msg = r"Number of elements in density \([0-9]+\) mismatch the number of prisms \([0-9]+\)"
    with pytest.raises(ValueError, match=msg):
        hg.prism_gravity([0, 0, 0], prisms, [1000, 2000], field="potential")


def test_invalid_prisms():
    """test/test_prism.py:73-91"""
    w, e, s, n, bottom, top = -100, 100, -100, 100, -200, -100
    hg.check_prisms(np.atleast_2d([w, e, s, n, bottom, top]))
    hg.check_prisms(np.atleast_2d([w, w, s, n, bottom, top]))
    hg.check_prisms(np.atleast_2d([w, e, s, s, bottom, top]))
    hg.check_prisms(np.atleast_2d([w, e, s, n, bottom, bottom]))
    with pytest.raises(ValueError, match="The west boundary can't be greater than the east one"):
        hg.check_prisms(np.atleast_2d([e, w, s, n, bottom, top]))
    with pytest.raises(ValueError, match="The south boundary can't be greater than the north one"):
        hg.check_prisms(np.atleast_2d([w, e, n, s, bottom, top]))
    with pytest.raises(ValueError, match="The bottom boundary can't be greater than the top one"):
        hg.check_prisms(np.atleast_2d([w, e, s, n, top, bottom]))


def test_invalid_prism_raises_before_gpu():
    with pytest.raises(ValueError, match="The bottom boundary can't be greater than the top one"):
        hg.prism_gravity([0, 0, 0], [0, 10, 0, 10, 0, -10], 100, field="potential")


@pytest.fixture
def dummy_layer():
    """test/test_prism_layer.py:33-49 (numpy variant)."""
    easting = np.linspace(-1, 3, 5)
    northing = np.linspace(7, 13, 4)
    shape = (northing.size, easting.size)
    surface = np.arange(20, dtype=float).reshape(*shape)
    density = 2670 * np.ones(shape)
    return (easting, northing), surface, 0, density


def test_prism_layer(dummy_layer):
    """test/test_prism_layer.py:79-106"""
    (easting, northing), surface, reference, _ = dummy_layer
    layer = hg.prism_layer((easting, northing), surface, reference)
    for name in ("easting", "northing", "top", "bottom"):
        assert name in layer.coords
    npt.assert_allclose(layer.easting, easting)
    npt.assert_allclose(layer.northing, northing)
    npt.assert_allclose(layer.top, surface)
    npt.assert_allclose(layer.bottom, reference)
    surface[1, 1] = -1
    expected_top = surface.copy()
    expected_bottom = np.zeros_like(surface)
    expected_top[1, 1], expected_bottom[1, 1] = reference, surface[1, 1]
    layer = hg.prism_layer((easting, northing), surface, reference)
    npt.assert_allclose(layer.top, expected_top)
    npt.assert_allclose(layer.bottom, expected_bottom)


def test_prism_layer_invalid_surface_reference(dummy_layer):
    """test/test_prism_layer.py:109-134"""
    coordinates, surface, reference, _ = dummy_layer
    msg = (
        r"Invalid surface array with shape '.+'\. "
        "Its shape should be compatible with the coordinates "
        r"of the layer of prisms\."
    )
    with pytest.raises(ValueError, match=msg):
        hg.prism_layer(coordinates, np.arange(20, dtype=float), reference)
    msg = msg.replace("surface", "reference")
    with pytest.raises(ValueError, match=msg):
        hg.prism_layer(coordinates, np.arange(20, dtype=float).reshape(4, 5), np.zeros(20))


def test_prism_layer_properties(dummy_layer):
    """test/test_prism_layer.py:137-150"""
    coordinates, surface, reference, density = dummy_layer
    sus = 0 * density + 1e-3
    layer = hg.prism_layer(
        coordinates, surface, reference, properties={"density": density, "suceptibility": sus}
    )
    npt.assert_allclose(layer.density, density)
    npt.assert_allclose(layer.suceptibility, sus)


def test_prism_layer_no_regular_grid(dummy_layer):
    """test/test_prism_layer.py:153-180"""
    (easting, northing), surface, reference, _ = dummy_layer
    easting_invalid = easting.copy()
    easting_invalid[3] = -22
    with pytest.raises(ValueError, match="Passed easting coordinates are not evenly spaced"):
        hg.prism_layer((easting_invalid, northing), surface, reference)
    northing_invalid = northing.copy()
    northing_invalid[3] = -22
    with pytest.raises(ValueError, match="Passed northing coordinates are not evenly spaced"):
        hg.prism_layer((easting, northing_invalid), surface, reference)


def test_prism_layer_attributes():
    """test/test_prism_layer.py:183-201"""
    easting = np.linspace(1, 3, 5)
    northing = np.linspace(7, 10, 4)
    layer = hg.prism_layer((easting, northing), np.arange(20, dtype=float).reshape(4, 5), 0)
    assert layer.prism_layer.dims == ("northing", "easting")
    assert layer.prism_layer.spacing == (1, 0.5)
    assert layer.prism_layer.boundaries == (
        easting[0] - 0.25, easting[-1] + 0.25, northing[0] - 0.5, northing[-1] + 0.5,
    )
    assert layer.prism_layer.size == 20
    assert layer.prism_layer.shape == (4, 5)


def test_prism_layer_to_prisms_and_get_prism():
    """test/test_prism_layer.py:204-237"""
    coordinates = (np.array([0, 1]), np.array([0, 1]))
    reference = np.arange(4).reshape(2, 2)
    surface = (np.arange(4) + 10).reshape(2, 2)
    layer = hg.prism_layer(coordinates, surface, reference)
    expected = [
        [-0.5, 0.5, -0.5, 0.5, 0, 10],
        [0.5, 1.5, -0.5, 0.5, 1, 11],
        [-0.5, 0.5, 0.5, 1.5, 2, 12],
        [0.5, 1.5, 0.5, 1.5, 3, 13],
    ]
    npt.assert_allclose(expected, layer.prism_layer._to_prisms())
    for i in range(2):
        for j in range(2):
            npt.assert_allclose(layer.prism_layer.get_prism((i, j)), expected[2 * i + j])


def test_layer_doctest_vectors():
    """Boundaries and get_prism printed by harmonica's doctest (layer.py:95-118)."""
    import json
    import os

    gold = json.load(
        open(os.path.join(os.path.dirname(__file__), "golden", "reference_doctests.json"))
    )["layer"]
    easting = np.linspace(0, 10, 5)
    northing = np.linspace(2, 8, 4)
    surface = np.arange(20, dtype=float).reshape((4, 5))
    layer = hg.prism_layer(
        (easting, northing), surface, reference=0, properties={"density": 2670.0 * np.ones((4, 5))}
    )
    assert [float(b) for b in layer.prism_layer.boundaries] == gold["boundaries"]
    assert [float(b) for b in layer.prism_layer.get_prism((0, 2))] == gold["get_prism_0_2"]


def test_layer_invalid_field(dummy_layer):
    """test/test_prism_layer.py:264-279"""
    coordinates, surface, reference, density = dummy_layer
    layer = hg.prism_layer(coordinates, surface, reference, properties={"density": density})
    msg = re.escape("Gravitational field 'invalid field' not recognized.")
    with pytest.raises(ValueError, match=msg):
        layer.prism_layer.gravity((0, 0, 0), field="invalid field")


def test_device_layer_exported():
    """The device-resident layer API is part of the package (GPU behaviour in
    test_gpu_device_layer.py)."""
    import harmonica_gb300 as hg

    assert callable(hg.prism_layer_device)
    assert hasattr(hg.DevicePrismLayer, "update_top_bottom")
    assert hasattr(hg.DevicePrismLayer, "gravity")
