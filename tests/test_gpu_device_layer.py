"""
Device-resident layer (prism_layer_device): top/bottom on the GPU equal the
host accessor's update_top_bottom (NaN surfaces and scalar/array references
included, layer.py:264-312), and its gravity equals the host layer's
accessor, for every field; the boundaries and prism rows agree too.
"""

import numpy as np
import numpy.testing as npt
import pytest

import harmonica_gb300 as hg

pytestmark = pytest.mark.gpu


def _grids(seed, shape=(23, 31)):
    rng = np.random.default_rng(seed)
    easting = np.linspace(0, 30e3, shape[1])
    northing = np.linspace(-5e3, 17e3, shape[0])
    surface = rng.uniform(-800, 1200, shape)
    surface[3, 4] = np.nan
    reference = rng.uniform(-300, 300, shape)
    density = rng.uniform(1800, 3000, shape)
    return easting, northing, surface, reference, density


@pytest.mark.parametrize("scalar_reference", [True, False])
def test_top_bottom_match_host(gpu_lib, scalar_reference):
    import torch

    easting, northing, surface, reference, density = _grids(1)
    ref = 100.0 if scalar_reference else reference
    dev = hg.prism_layer_device((easting, northing), surface, ref, properties={"density": density})
    host = hg.prism_layer((easting, northing), surface, ref, properties={"density": density})
    npt.assert_array_equal(dev.top.cpu().numpy(), np.asarray(host.top.values))
    npt.assert_array_equal(dev.bottom.cpu().numpy(), np.asarray(host.bottom.values))
    assert isinstance(dev.top, torch.Tensor) and dev.top.is_cuda
    acc = hg.DatasetAccessorPrismLayer(host)
    assert dev.shape == acc.shape and dev.size == acc.size
    npt.assert_allclose(dev.spacing, acc.spacing)
    npt.assert_allclose(dev.boundaries, acc.boundaries)
    npt.assert_array_equal(dev.to_prisms().cpu().numpy(), acc._to_prisms())


@pytest.mark.parametrize("field", ["g_z", "potential", "g_e", "g_zz", "g_nz"])
def test_gravity_matches_host_layer(gpu_lib, field):
    import torch

    easting, northing, surface, reference, density = _grids(2)
    density[5, 6] = 0.0
    dev = hg.prism_layer_device((easting, northing), surface, reference,
                                properties={"density": density})
    host = hg.prism_layer((easting, northing), surface, reference,
                          properties={"density": density})
    e, n = np.meshgrid(np.linspace(-2e3, 32e3, 17), np.linspace(-7e3, 19e3, 13))
    u = np.full_like(e, 1500.0)
    got = dev.gravity((e, n, u), field, thickness_threshold=1.0)
    assert isinstance(got, torch.Tensor) and got.is_cuda and tuple(got.shape) == e.shape
    ref = hg.DatasetAccessorPrismLayer(host).gravity((e, n, u), field, thickness_threshold=1.0)
    npt.assert_array_equal(got.cpu().numpy(), ref)


def test_nan_density_warns(gpu_lib):
    easting, northing, surface, reference, density = _grids(4)
    density[1, 1] = np.nan
    dev = hg.prism_layer_device((easting, northing), surface, reference,
                                properties={"density": density})
    with pytest.warns(UserWarning, match="NaN values in 'density'"):
        dev.gravity(([1e3], [2e3], [3e3]), "g_z")


def test_update_in_place_loop_stays_on_device(gpu_lib):
    import torch

    easting, northing, surface, reference, density = _grids(3)
    dev = hg.prism_layer_device((easting, northing), surface, reference,
                                properties={"density": density})
    e = torch.linspace(0, 30e3, 50, dtype=torch.float64, device=dev.device)
    n = torch.zeros_like(e)
    u = torch.full_like(e, 2000.0)
    first = dev.gravity((e, n, u), "g_z", check_nan=False)
    dev.update_top_bottom(dev.top + 10.0, torch.as_tensor(reference, device=dev.device))
    second = dev.gravity((e, n, u), "g_z", check_nan=False)
    assert second.is_cuda and bool((second != first).any())
    with pytest.raises(ValueError, match="Invalid surface"):
        dev.update_top_bottom(np.zeros((2, 2)), 0.0)
