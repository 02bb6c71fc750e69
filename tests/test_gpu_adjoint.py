"""
Adjoint kernels behind torch.autograd: gradients of a weighted sum of the
forward (any field for densities, g_z for bottoms/tops) against
(1) gradients assembled from single-prism forward calls of the CPU oracle and
(2) central finite differences (h = 1e-2 m, 1e-3 kg/m^3) of single-prism
oracle forwards.  Tolerance: 1e-9 relative for the linear density gradient,
1e-6 relative for the geometric (finite-difference) gradients.
"""

import numpy as np
import numpy.testing as npt
import pytest

import harmonica_gb300 as hg
from harmonica_gb300 import synthetic

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def small_basement():
    L = synthetic.basement_layer(n_side=24, spacing=500.0, n_stations_side=15)
    rng = np.random.default_rng(L["noise_seed"])
    # dL/dd_i: positive weights, so that the weighted finite differences of
    # single prisms below do not cancel (a signed residual makes the weighted
    # sum ~100x smaller than its terms and the FD reference noisier than 1e-6)
    w = rng.uniform(0.5, 1.5, L["coordinates"][0].size)
    return L, w


def _layer_prisms(L):
    return synthetic.layer_to_prisms(L)


def test_layer_adjoint_density_and_geometry(gpu_lib, oracle, small_basement):
    import torch

    L, w = small_basement
    dev = torch.device("cuda")
    T = lambda a: torch.tensor(a, dtype=torch.float64, device=dev)  # noqa: E731
    rho = T(L["density"]).requires_grad_(True)
    bot = T(L["bottom"]).requires_grad_(True)
    top = T(L["top"]).requires_grad_(True)
    coords = tuple(T(c) for c in L["coordinates"])
    gz = hg.layer_gravity_torch(coords, T(L["easting"]), T(L["northing"]), bot, top, rho)
    # forward equals the oracle layer forward
    ref = oracle.layer_gravity(L["coordinates"], L["easting"], L["northing"], L["bottom"],
                               L["top"], L["density"], "g_z")
    npt.assert_allclose(gz.detach().cpu().numpy(), ref, rtol=1e-8,
                        atol=1e-9 * np.abs(ref).max())
    (gz * T(w)).sum().backward()
    g_rho = rho.grad.cpu().numpy().ravel()
    g_bot = bot.grad.cpu().numpy().ravel()
    g_top = top.grad.cpu().numpy().ravel()
    prisms, dens = _layer_prisms(L)
    rng = np.random.default_rng(0)
    for j in rng.choice(prisms.shape[0], 6, replace=False):
        p = prisms[j]
        k = oracle.prism_gravity(L["coordinates"], [p], [1.0], "g_z")
        npt.assert_allclose(g_rho[j], np.dot(w, k), rtol=1e-9)
        h = 1e-2
        for col, g in ((4, g_bot), (5, g_top)):
            pp, pm = p.copy(), p.copy()
            pp[col] += h
            pm[col] -= h
            fd = (oracle.prism_gravity(L["coordinates"], [pp], [dens[j]], "g_z")
                  - oracle.prism_gravity(L["coordinates"], [pm], [dens[j]], "g_z")) / (2 * h)
            npt.assert_allclose(g[j], np.dot(w, fd), rtol=1e-6)


@pytest.mark.parametrize("field", hg.FIELDS)
def test_prism_adjoint_density_all_fields(gpu_lib, oracle, field):
    import torch

    rng = np.random.default_rng(3)
    m, n = 40, 60
    west = rng.uniform(-2e3, 2e3, m)
    south = rng.uniform(-2e3, 2e3, m)
    top = rng.uniform(-300, 0, m)
    horiz = np.column_stack([west, west + rng.uniform(50, 500, m), south,
                             south + rng.uniform(50, 500, m)])
    bottom = top - rng.uniform(50, 800, m)
    rho = rng.uniform(-500, 500, m)
    coords = (rng.uniform(-2.5e3, 2.5e3, n), rng.uniform(-2.5e3, 2.5e3, n),
              rng.uniform(10, 300, n))
    w = rng.normal(size=n)
    dev = torch.device("cuda")
    T = lambda a: torch.tensor(a, dtype=torch.float64, device=dev)  # noqa: E731
    trho = T(rho).requires_grad_(True)
    out = hg.prism_gravity_torch(tuple(T(c) for c in coords), T(horiz), T(bottom), T(top), trho,
                                 field=field)
    (out * T(w)).sum().backward()
    g = trho.grad.cpu().numpy()
    prisms = np.column_stack([horiz, bottom, top])
    expected = np.array([np.dot(w, oracle.prism_gravity(coords, [prisms[j]], [1.0], field))
                         for j in range(m)])
    npt.assert_allclose(g, expected, rtol=1e-9, atol=1e-12 * np.abs(expected).max())


def test_prism_adjoint_geometry_gz_finite_differences(gpu_lib, oracle):
    import torch

    rng = np.random.default_rng(4)
    m, n = 25, 50
    west = rng.uniform(-1e3, 1e3, m)
    south = rng.uniform(-1e3, 1e3, m)
    horiz = np.column_stack([west, west + 300.0, south, south + 250.0])
    top = rng.uniform(-200, 0, m)
    bottom = top - rng.uniform(100, 1500, m)
    rho = rng.uniform(-500, 500, m)
    coords = (rng.uniform(-1.5e3, 1.5e3, n), rng.uniform(-1.5e3, 1.5e3, n),
              rng.uniform(50, 500, n))
    w = rng.normal(size=n)
    dev = torch.device("cuda")
    T = lambda a: torch.tensor(a, dtype=torch.float64, device=dev)  # noqa: E731
    tb, tt = T(bottom).requires_grad_(True), T(top).requires_grad_(True)
    out = hg.prism_gravity_torch(tuple(T(c) for c in coords), T(horiz), tb, tt, T(rho))
    (out * T(w)).sum().backward()
    prisms = np.column_stack([horiz, bottom, top])
    h = 1e-2
    for j in range(m):
        for col, g in ((4, tb.grad), (5, tt.grad)):
            pp, pm = prisms[j].copy(), prisms[j].copy()
            pp[col] += h
            pm[col] -= h
            fd = (oracle.prism_gravity(coords, [pp], [rho[j]], "g_z")
                  - oracle.prism_gravity(coords, [pm], [rho[j]], "g_z")) / (2 * h)
            npt.assert_allclose(g[j].item(), np.dot(w, fd), rtol=1e-6)


def test_density_gradient_matches_finite_difference_of_gpu_forward(gpu_lib):
    """Central FD (1e-3 kg/m^3) of the GPU misfit itself for a few densities.

    The misfit difference is ~1e-2 while each misfit carries the forward's
    ~1e-12 relative rounding through ~1e2 stations, so this end-to-end FD is
    checked at 1e-5; the 1e-6 checks above difference single prisms."""
    import torch

    L = synthetic.basement_layer(n_side=16, spacing=500.0, n_stations_side=10)
    dev = torch.device("cuda")
    T = lambda a: torch.tensor(a, dtype=torch.float64, device=dev)  # noqa: E731
    coords = tuple(T(c) for c in L["coordinates"])
    data = np.random.default_rng(1).normal(0, 0.1, L["coordinates"][0].size)

    def misfit(rho):
        gz = hg.layer_gravity_torch(coords, T(L["easting"]), T(L["northing"]), T(L["bottom"]),
                                    T(L["top"]), rho)
        return 0.5 * ((gz - T(data)) ** 2).sum()

    rho = T(L["density"]).requires_grad_(True)
    misfit(rho).backward()
    g = rho.grad.cpu().numpy()
    h = 1e-3
    for (a, b) in ((0, 0), (7, 9), (15, 3)):
        rp = T(L["density"]).clone()
        rm = T(L["density"]).clone()
        rp[a, b] += h
        rm[a, b] -= h
        fd = (misfit(rp) - misfit(rm)).item() / (2 * h)
        npt.assert_allclose(g[a, b], fd, rtol=1e-5)
