"""
Array sizes are checked on the host before any kernel reads them, even with
``disable_checks=True``: the C ABI receives bare pointers, so a short array
would otherwise be read past its end on the device.  Every case here raises
``ValueError`` before a device is touched, so these run on CPU.
"""

import numpy as np
import pytest
import torch

import harmonica_gb300 as hg
from harmonica_gb300.equivalent_sources import greens_jacobian, greens_predict
from harmonica_gb300.gravity import forward_on_device, pack_prisms
from harmonica_gb300.layer import layer_forward_device

COORDS = ([0.0, 10.0], [0.0, 5.0], [100.0, 100.0])
PRISMS = [[-10, 10, -10, 10, -20, -10], [20, 30, 20, 30, -20, -10]]


@pytest.mark.parametrize("disable_checks", [False, True])
def test_prism_density_count(disable_checks):
    with pytest.raises(ValueError, match=r"Number of elements in density \(1\) mismatch"):
        hg.prism_gravity(COORDS, PRISMS, [2670.0], "g_z", disable_checks=disable_checks)


@pytest.mark.parametrize("disable_checks", [False, True])
def test_prism_columns(disable_checks):
    with pytest.raises(ValueError, match="six"):
        hg.prism_gravity(COORDS, [[0, 1, 0, 1, -1]], [1.0], "g_z", disable_checks=disable_checks)


@pytest.mark.parametrize("disable_checks", [False, True])
def test_magnetization_components(disable_checks):
    with pytest.raises(ValueError, match=r"Number of magnetization vectors \(1\) mismatch"):
        hg.prism_magnetic(COORDS, PRISMS, ([1.0, 1.0], [1.0, 1.0], [1.0]), "b_u",
                          disable_checks=disable_checks)
    with pytest.raises(ValueError, match="with '2' elements"):
        hg.prism_magnetic(COORDS, PRISMS, ([1.0, 1.0], [1.0, 1.0]), "b_u",
                          disable_checks=disable_checks)


def test_point_mass_coordinates():
    with pytest.raises(ValueError, match="same number of elements"):
        hg.point_gravity(COORDS, ([0.0, 1.0], [0.0, 1.0], [-10.0]), [1.0, 2.0], "g_z")


@pytest.mark.parametrize("disable_checks", [False, True])
def test_dipole_coordinates(disable_checks):
    with pytest.raises(ValueError, match="same number of elements"):
        hg.dipole_magnetic(COORDS, ([0.0, 1.0], [0.0], [-10.0, -10.0]),
                           ([1.0, 1.0], [1.0, 1.0], [1.0, 1.0]), "b_u",
                           disable_checks=disable_checks)


@pytest.mark.parametrize("disable_checks", [False, True])
def test_tesseroid_columns(disable_checks):
    with pytest.raises(ValueError, match="six"):
        hg.tesseroid_gravity(([0.0], [0.0], [6.4e6]), np.zeros((4, 3)), np.ones(4), "g_z",
                             disable_checks=disable_checks)


def test_equivalent_source_sizes():
    with pytest.raises(ValueError, match="sources"):
        greens_jacobian(COORDS, ([0.0, 1.0], [0.0], [-10.0, -10.0]))
    with pytest.raises(ValueError, match="data points"):
        greens_jacobian(([0.0, 1.0], [0.0], [1.0, 1.0]), ([0.0], [0.0], [-10.0]))
    with pytest.raises(ValueError, match=r"coefficients \(1\) mismatch the number of sources"):
        greens_predict(COORDS, ([0.0, 1.0], [0.0, 1.0], [-10.0, -10.0]), [1.0])


def _f64(*values):
    return torch.tensor(values, dtype=torch.float64)


def test_layer_grid_sizes():
    e, n, u = _f64(0.0), _f64(0.0), _f64(10.0)
    ce, cn = _f64(0.0, 1.0, 2.0), _f64(0.0, 1.0)
    full = torch.zeros(6, dtype=torch.float64)
    short = torch.zeros(5, dtype=torch.float64)
    for bottom, top, density, name in ((short, full, full, "bottom"),
                                       (full, short, full, "top"),
                                       (full, full, short, "density")):
        with pytest.raises(ValueError, match=f"Invalid '{name}' with 5 values"):
            layer_forward_device(e, n, u, ce, cn, bottom, top, density, 1 << 3, 0.0)
    with pytest.raises(ValueError, match="observation points"):
        layer_forward_device(_f64(0.0, 1.0), n, u, ce, cn, full, full, full, 1 << 3, 0.0)


def test_device_helpers_check_shapes_and_layout():
    prisms = torch.zeros((2, 6), dtype=torch.float64)
    with pytest.raises(ValueError, match="M densities"):
        pack_prisms(prisms, _f64(1.0))
    with pytest.raises(ValueError, match="contiguous float64"):
        pack_prisms(prisms.float(), _f64(1.0, 2.0))
    with pytest.raises(ValueError, match="contiguous float64"):
        pack_prisms(torch.zeros((6, 2), dtype=torch.float64).T, _f64(1.0, 2.0))
    e = _f64(0.0, 1.0)
    with pytest.raises(ValueError, match="observation points"):
        forward_on_device(e, _f64(0.0), e, torch.zeros((7, 2), dtype=torch.float64), 2, 1 << 3)
    with pytest.raises(ValueError, match=r"\(7, >= 3\)"):
        forward_on_device(e, e, e, torch.zeros((7, 2), dtype=torch.float64), 3, 1 << 3)


def test_device_layer_property_shapes():
    from harmonica_gb300.device_layer import DevicePrismLayer

    easting, northing = _f64(0.0, 1.0, 2.0), _f64(0.0, 1.0)
    ok = {"density": torch.zeros((2, 3), dtype=torch.float64)}
    assert DevicePrismLayer(easting, northing, ok, "cpu").shape == (2, 3)
    bad = {"density": torch.zeros((3, 2), dtype=torch.float64)}
    with pytest.raises(ValueError, match="Invalid property 'density'"):
        DevicePrismLayer(easting, northing, bad, "cpu")


def test_host_layer_property_shapes():
    easting, northing = np.linspace(0, 20, 3), np.linspace(0, 10, 2)
    surface = np.ones((2, 3))
    layer = hg.prism_layer((easting, northing), surface, 0.0,
                           properties={"density": np.ones((2, 3))})
    assert layer.prism_layer.shape == (2, 3)
    with pytest.raises(ValueError, match="Invalid property 'density'"):
        hg.prism_layer((easting, northing), surface, 0.0, properties={"density": np.ones((3, 2))})


def test_tesseroid_device_entry_checks_sizes_and_layout():
    from harmonica_gb300.tesseroid import tesseroid_gravity_device

    pts = _f64(0.0, 1.0)
    tess = torch.zeros((3, 6), dtype=torch.float64)
    with pytest.raises(ValueError, match="same number of elements"):
        tesseroid_gravity_device(pts, _f64(0.0), pts, tess, torch.zeros(3, dtype=torch.float64),
                                 "g_z")
    with pytest.raises(ValueError, match=r"density must have shape \(3,\) or \(3, 2\)"):
        tesseroid_gravity_device(pts, pts, pts, tess, torch.zeros(2, dtype=torch.float64), "g_z")
    with pytest.raises(ValueError, match=r"\(M, 6\)"):
        tesseroid_gravity_device(pts, pts, pts, torch.zeros((3, 5), dtype=torch.float64),
                                 torch.zeros(3, dtype=torch.float64), "g_z")
    with pytest.raises(ValueError, match="contiguous float64"):
        tesseroid_gravity_device(pts.float(), pts, pts, tess, torch.zeros(3, dtype=torch.float64),
                                 "g_z")
    with pytest.raises(ValueError, match="status"):
        tesseroid_gravity_device(pts, pts, pts, tess, torch.zeros(3, dtype=torch.float64), "g_z",
                                 status=torch.zeros(1, dtype=torch.int64))


def test_tesseroid_layer_property_shapes():
    longitude, latitude = np.linspace(-10, 10, 5), np.linspace(-5, 5, 3)
    surface = np.full((3, 5), 6.371e6)
    layer = hg.tesseroid_layer((longitude, latitude), surface, 6.36e6,
                               properties={"density": np.ones((3, 5))})
    assert layer.tesseroid_layer.shape == (3, 5)
    with pytest.raises(ValueError, match="Invalid property 'density'"):
        hg.tesseroid_layer((longitude, latitude), surface, 6.36e6,
                           properties={"density": np.ones((5, 3))})
