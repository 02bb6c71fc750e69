"""
Prism-layer accessor on the GPU: harmonica's test/test_prism_layer.py
behaviour (accessor == prism_gravity of _to_prisms, NaN holes, density NaN
warning, thickness threshold) and parity with the layer oracle, including
the 1e4-prism topography layer at full size.
"""

import re
import warnings

import numpy as np
import numpy.testing as npt
import pytest

import harmonica_gb300 as hg
from harmonica_gb300 import synthetic

pytestmark = pytest.mark.gpu

FIELDS = hg.FIELDS


def assert_parity(actual, expected, rtol=1e-8, atol_frac=1e-9, msg=""):
    expected = np.asarray(expected)
    fin = np.isfinite(expected)
    atol = atol_frac * (np.abs(expected[fin]).max() if fin.any() else 0.0)
    npt.assert_array_equal(np.isnan(actual), np.isnan(expected), err_msg=msg)
    npt.assert_allclose(np.asarray(actual)[fin], expected[fin], rtol=rtol, atol=atol, err_msg=msg)


@pytest.fixture
def dummy_layer():
    """test/test_prism_layer.py:33-49"""
    easting = np.linspace(-1, 3, 5)
    northing = np.linspace(7, 13, 4)
    shape = (northing.size, easting.size)
    surface = np.arange(20, dtype=float).reshape(*shape)
    density = 2670 * np.ones(shape)
    return (easting, northing), surface, 0, density


def grid_coords():
    e, n = np.meshgrid(np.arange(1, 3.5, 1.0), np.arange(7, 10.5, 1.0))
    return (e, n, np.full_like(e, 30.0))


@pytest.mark.parametrize("field", FIELDS)
def test_layer_gravity_matches_prism_gravity(gpu_lib, dummy_layer, field):
    """test/test_prism_layer.py:240-261"""
    coords = grid_coords()
    (easting, northing), surface, reference, density = dummy_layer
    layer = hg.prism_layer((easting, northing), surface, reference,
                           properties={"density": density})
    expected = hg.prism_gravity(coords, layer.prism_layer._to_prisms(), density, field=field)
    npt.assert_allclose(expected, layer.prism_layer.gravity(coords, field=field), rtol=1e-10)


def test_layer_progress_bar(gpu_lib, dummy_layer):
    """test/test_prism_layer.py:401-419: the accessor's results with and
    without the progress bar match."""
    e, n = np.meshgrid(np.arange(1, 4, 1.0), np.arange(7, 11, 1.0))
    coords = (e, n, np.full_like(e, 30.0))
    (easting, northing), surface, reference, density = dummy_layer
    layer = hg.prism_layer((easting, northing), surface, reference,
                           properties={"density": density})
    npt.assert_allclose(layer.prism_layer.gravity(coords, field="g_z", progressbar=True),
                        layer.prism_layer.gravity(coords, field="g_z", progressbar=False))


def _holes(dummy_layer):
    (easting, northing), surface, reference, density = dummy_layer
    layer = hg.prism_layer((easting, northing), surface, reference,
                           properties={"density": density})
    idx = [(3, 3), (2, 1)]
    prisms = [layer.prism_layer.get_prism((i, j)) for i in range(4) for j in range(5)
              if (i, j) not in idx]
    rho = [density[i, j] for i in range(4) for j in range(5) if (i, j) not in idx]
    return idx, prisms, rho


@pytest.mark.parametrize("field", ["potential", "g_z"])
def test_layer_surface_nans(gpu_lib, dummy_layer, field):
    """test/test_prism_layer.py:282-304"""
    coords = grid_coords()
    (easting, northing), surface, reference, density = dummy_layer
    idx, prisms, rho = _holes(dummy_layer)
    surface = surface.copy()
    for index in idx:
        surface[index] = np.nan
    layer = hg.prism_layer((easting, northing), surface, reference,
                           properties={"density": density})
    npt.assert_allclose(layer.prism_layer.gravity(coords, field=field),
                        hg.prism_gravity(coords, prisms, rho, field=field), rtol=1e-10)


@pytest.mark.parametrize("field", ["potential", "g_z"])
def test_layer_density_nans(gpu_lib, dummy_layer, field):
    """test/test_prism_layer.py:307-334"""
    coords = grid_coords()
    (easting, northing), surface, reference, density = dummy_layer
    idx, prisms, rho = _holes(dummy_layer)
    density = density.copy()
    for index in idx:
        density[index] = np.nan
    layer = hg.prism_layer((easting, northing), surface, reference,
                           properties={"density": density})
    msg = re.escape("Found NaN values in 'density' property of the prisms layer.")
    with pytest.warns(match=msg):
        result = layer.prism_layer.gravity(coords, field=field)
    npt.assert_allclose(result, hg.prism_gravity(coords, prisms, rho, field=field), rtol=1e-10)


def test_layer_thickness_threshold(gpu_lib, dummy_layer):
    """test/test_prism_layer.py:422-456"""
    coords = grid_coords()
    prism_coords, surface, reference, density = dummy_layer
    layer = hg.prism_layer(prism_coords, surface, reference, properties={"density": density})
    npt.assert_allclose(layer.prism_layer.gravity(coords, field="g_z"),
                        layer.prism_layer.gravity(coords, field="g_z", thickness_threshold=0))
    kept = [p for p in layer.prism_layer._to_prisms() if abs(p[5] - p[4]) >= 5.0]
    npt.assert_allclose(
        hg.prism_gravity(coords, kept, [2670] * len(kept), field="g_z"),
        layer.prism_layer.gravity(coords, field="g_z", thickness_threshold=5),
        rtol=1e-10,
    )


@pytest.mark.parametrize("field", FIELDS)
def test_layer_against_oracle_golden(gpu_lib, field):
    import os

    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "oracle_small.npz"))
    layer = hg.prism_layer((g["layer_easting"], g["layer_northing"]), g["layer_top"],
                           g["layer_bottom"], properties={"density": g["layer_density"]})
    coords = (g["layer_obs_e"], g["layer_obs_n"], g["layer_obs_u"])
    assert_parity(layer.prism_layer.gravity(coords, field=field), g[f"layer_{field}"], msg=field)


def test_topography_1e4_full_size_against_oracle(gpu_lib, oracle):
    """The 100 x 100-prism layer with 50 x 50 stations, all 2.5e7 pairs, g_z."""
    L = synthetic.layer_topography_1e4()
    layer = hg.prism_layer((L["easting"], L["northing"]), L["top"], L["bottom"],
                           properties={"density": L["density"]})
    res = layer.prism_layer.gravity(L["coordinates"], field="g_z")
    ref = oracle.layer_gravity(L["coordinates"], L["easting"], L["northing"], L["bottom"],
                               L["top"], L["density"], "g_z")
    assert_parity(res, ref, msg="g_z")


def test_topography_1e6_subset_against_oracle(gpu_lib, oracle):
    """The 1000 x 1000-prism layer (all 1e6 prisms) on 256 of its stations,
    all ten fields, through the accessor (single-field kernels) and the fused
    all-field layer launch, against the oracle's layer loop."""
    from harmonica_gb300.layer import layer_forward

    L = synthetic.layer_topography_1e6()
    rng = np.random.default_rng(0)
    idx = rng.choice(L["coordinates"][0].size, 256, replace=False)
    coords = tuple(c[idx] for c in L["coordinates"])
    layer = hg.prism_layer((L["easting"], L["northing"]), L["top"], L["bottom"],
                           properties={"density": L["density"]})
    ref = oracle.layer_gravity_fields(coords, L["easting"], L["northing"], L["bottom"],
                                      L["top"], L["density"])
    fused = layer_forward(coords, L["easting"], L["northing"], L["bottom"], L["top"],
                          L["density"], 0x3FF, 0.0)
    for code, field in enumerate(hg.FIELDS):
        assert_parity(layer.prism_layer.gravity(coords, field=field), ref[field], msg=field)
        assert_parity(fused[code], ref[field], msg=f"{field} fused")


def test_layer_no_singular_warning(gpu_lib, dummy_layer):
    """The accessor does not scan for singular points (layer.py:314-433)."""
    (easting, northing), surface, reference, density = dummy_layer
    layer = hg.prism_layer((easting, northing), surface, reference + 0.5,
                           properties={"density": density})
    w, e, s, n, b, t = layer.prism_layer.get_prism((1, 1))
    with warnings.catch_warnings():
        warnings.simplefilter("error")
        v = layer.prism_layer.gravity((w, s, b), field="g_zz")
    assert np.isnan(v)
