"""
The basement-inversion step at its full size: a 200 x 200 layer of 500 m
cells (tops at 0 m, smooth bottoms N(-3000, 800) m, contrast -400 kg/m^3),
g_z on 100 x 100 stations at 500 m, an L2 misfit against the true model's
data plus N(0, 0.1 mGal) noise, evaluated at a flat -3000 m starting model
(the first step of an inversion).  The forward and both gradients are
checked on the full problem:

* forward: against the CPU oracle on a strided sample of 400 stations
  (1e-8 relative, 1e-9 x max absolute);
* d misfit / d density: against the residual-weighted sum of the oracle's
  single-prism forwards over all 10,000 stations (the gradient is linear in
  the forward; 1e-9 relative), and against central differences of the GPU
  misfit at h = 1e-3 kg/m^3;
* d misfit / d bottom: against central differences of the GPU misfit at
  h = 1e-2 m.

Tolerance of the misfit differences.  Moving one parameter changes one
prism's term of the forward; every other term is evaluated bitwise the same,
so the difference of two misfits carries only that term's rounding and the
rounding of each station's running sum (~1e-16 of |g_z|, ~2e-14 mGal) times
the residuals (~10 mGal) over 10,000 stations: ~1e-9 absolute.  The density
differences (misfit change ~1e-1) are checked at 1e-6 relative; the bottom
differences (misfit change ~1e-4, a second-order truncation of (h / 500 m)^2
~ 4e-10) at 1e-5.
"""

import numpy as np
import numpy.testing as npt
import pytest

import harmonica_gb300 as hg
from harmonica_gb300 import synthetic

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def inversion():
    import torch

    L = synthetic.basement_layer()  # 200 x 200 cells, 100 x 100 stations
    dev = torch.device("cuda")
    T = lambda a: torch.tensor(a, dtype=torch.float64, device=dev)  # noqa: E731
    coords = tuple(T(c) for c in L["coordinates"])
    ce, cn = T(L["easting"]), T(L["northing"])
    with torch.no_grad():
        true_gz = hg.layer_gravity_torch(coords, ce, cn, T(L["bottom"]), T(L["top"]),
                                         T(L["density"]))
    rng = np.random.default_rng(L["noise_seed"])
    data = true_gz + T(rng.normal(0.0, 0.1, true_gz.numel()))
    start = np.full_like(L["bottom"], -3000.0)

    def misfit(bottom, density):
        with torch.no_grad():
            gz = hg.layer_gravity_torch(coords, ce, cn, T(bottom), T(L["top"]), T(density))
            return 0.5 * float(((gz - data) ** 2).sum())

    bottom = T(start).requires_grad_(True)
    rho = T(L["density"]).requires_grad_(True)
    gz = hg.layer_gravity_torch(coords, ce, cn, bottom, T(L["top"]), rho)
    resid = gz - data
    (0.5 * (resid ** 2).sum()).backward()
    return dict(L=L, start=start, gz=gz.detach().cpu().numpy(),
                resid=resid.detach().cpu().numpy(), g_bottom=bottom.grad.cpu().numpy(),
                g_density=rho.grad.cpu().numpy(), misfit=misfit)


def _prism(L, bottom, k):
    """Boundaries (w, e, s, n, b, t) of layer cell k (row-major over northing, easting)."""
    i, j = divmod(k, L["easting"].size)
    h = 250.0
    e0, n0 = L["easting"][j], L["northing"][i]
    return np.array([e0 - h, e0 + h, n0 - h, n0 + h, bottom.ravel()[k], L["top"].ravel()[k]])


def test_forward_full_size_against_oracle(gpu_lib, oracle, inversion):
    L, start = inversion["L"], inversion["start"]
    idx = np.arange(0, L["coordinates"][0].size, 25)  # 400 stations
    sample = tuple(c[idx] for c in L["coordinates"])
    ref = oracle.layer_gravity(sample, L["easting"], L["northing"], start, L["top"],
                               L["density"], "g_z")
    got = inversion["gz"][idx]
    npt.assert_allclose(got, ref, rtol=1e-8, atol=1e-9 * np.abs(ref).max())


def test_density_gradient_full_size(gpu_lib, oracle, inversion):
    L, start, resid = inversion["L"], inversion["start"], inversion["resid"]
    g = inversion["g_density"].ravel()
    rng = np.random.default_rng(11)
    cells = rng.choice(L["bottom"].size, 6, replace=False)
    for k in cells:
        kernel = oracle.prism_gravity(L["coordinates"], [_prism(L, start, k)], [1.0], "g_z")
        npt.assert_allclose(g[k], np.dot(resid, kernel), rtol=1e-9)
    misfit = inversion["misfit"]
    h = 1e-3
    for k in cells[:3]:
        rp = L["density"].copy()
        rm = L["density"].copy()
        rp.ravel()[k] += h
        rm.ravel()[k] -= h
        fd = (misfit(start, rp) - misfit(start, rm)) / (2 * h)
        npt.assert_allclose(g[k], fd, rtol=1e-6)


def test_bottom_gradient_full_size_central_differences(gpu_lib, inversion):
    L, start = inversion["L"], inversion["start"]
    g = inversion["g_bottom"].ravel()
    misfit = inversion["misfit"]
    rng = np.random.default_rng(12)
    h = 1e-2
    # interior cells (bottom and top stay apart by far more than h)
    for k in rng.choice(L["bottom"].size, 4, replace=False):
        bp = start.copy()
        bm = start.copy()
        bp.ravel()[k] += h
        bm.ravel()[k] -= h
        fd = (misfit(bp, L["density"]) - misfit(bm, L["density"])) / (2 * h)
        npt.assert_allclose(g[k], fd, rtol=1e-5)
