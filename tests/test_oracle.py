"""
Pin the CPU oracle before trusting it (no GPU needed).

* against the numbers harmonica prints in its own doctests
  (tests/golden/reference_doctests.json, from gravity.py:170-193);
* against an independent numerical quadrature of the defining integrals for
  all ten fields (this pins the formulas and the signs);
* against the behavioural tests of the reference test suite
  (test/test_prism.py: infinite slab :269-297, Laplace :247-266, null
  prisms :115-136, disable_checks :139-158, singular points :380-502);
* against a 50-digit mpmath evaluation of the same closed form.
"""

import json
import os
import warnings

import numpy as np
import numpy.testing as npt
import pytest

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
FIELDS = ("potential", "g_e", "g_n", "g_z", "g_ee", "g_nn", "g_zz", "g_en", "g_ez", "g_nz")


def test_reference_doctest_vectors(oracle):
    gold = json.load(open(os.path.join(GOLDEN, "reference_doctests.json")))
    coords = gold["coordinates"]
    for case in ("single_prism", "two_prisms"):
        c = gold[case]
        gz = oracle.prism_gravity(coords, c["prisms"], c["density"], field="g_z")
        npt.assert_allclose(np.round(gz, 5), c["g_z"], atol=0, rtol=0)


def test_golden_regression(oracle):
    g = np.load(os.path.join(GOLDEN, "oracle_small.npz"))
    coords = (g["choclo_e"], g["choclo_n"], g["choclo_u"])
    for f in FIELDS:
        npt.assert_allclose(
            oracle.prism_gravity(coords, g["choclo_prisms"], g["choclo_density"], f),
            g[f"choclo_{f}"],
            rtol=1e-13,
        )


def test_against_quadrature(oracle):
    integrate = pytest.importorskip("scipy.integrate")
    G = 6.6743e-11
    prism = np.array([-30.0, 50.0, -20.0, 40.0, -90.0, -35.0])
    rho = 2500.0
    P = np.array([12.0, -7.0, 15.0])

    def R(x, y, z):
        return np.sqrt(x * x + y * y + z * z)

    integrands = {
        "potential": lambda x, y, z: 1 / R(x, y, z),
        "g_e": lambda x, y, z: x / R(x, y, z) ** 3,
        "g_n": lambda x, y, z: y / R(x, y, z) ** 3,
        "g_z": lambda x, y, z: z / R(x, y, z) ** 3,
        "g_ee": lambda x, y, z: (3 * x * x - R(x, y, z) ** 2) / R(x, y, z) ** 5,
        "g_nn": lambda x, y, z: (3 * y * y - R(x, y, z) ** 2) / R(x, y, z) ** 5,
        "g_zz": lambda x, y, z: (3 * z * z - R(x, y, z) ** 2) / R(x, y, z) ** 5,
        "g_en": lambda x, y, z: 3 * x * y / R(x, y, z) ** 5,
        "g_ez": lambda x, y, z: 3 * x * z / R(x, y, z) ** 5,
        "g_nz": lambda x, y, z: 3 * y * z / R(x, y, z) ** 5,
    }
    for field, f in integrands.items():
        val, _ = integrate.tplquad(
            lambda z, y, x: f(x - P[0], y - P[1], z - P[2]),
            prism[0], prism[1], prism[2], prism[3], prism[4], prism[5],
            epsabs=0, epsrel=1e-11,
        )
        kern = oracle.prism_kernel(field, P, prism, rho)
        npt.assert_allclose(kern, G * rho * val, rtol=1e-9, err_msg=field)


def test_infinite_slab(oracle):
    """test/test_prism.py:269-297 with bouguer_correction (2 pi G rho h)."""
    height, thickness, density = 1.5, 10.5, 2670
    top, bottom = height, height - thickness
    sizes = np.logspace(3, 9, 7)
    results = np.array(
        [
            oracle.prism_gravity((0, 0, height), [-s / 2, s / 2, -s / 2, s / 2, bottom, top],
                                 density, "g_z")
            for s in sizes
        ]
    )
    analytical = 1e5 * 2 * np.pi * 6.6743e-11 * density * thickness
    errors = np.abs(analytical - results)
    assert (errors[1:] < errors[:-1]).all()
    npt.assert_allclose(analytical, results[-1], rtol=1e-7)


def test_laplace(oracle):
    """test/test_prism.py:247-266: g_ee + g_nn = -g_zz."""
    e, n = np.meshgrid(np.linspace(-10e3, 10e3, 10), np.linspace(-10e3, 10e3, 10))
    coords = (e, n, np.full_like(e, 300.0))
    prisms = [[1e3, 7e3, -5e3, 2e3, -1e3, -500], [-4e3, 1e3, 4e3, 10e3, -2e3, 200]]
    rho = [2670.0, 2900.0]
    d = {f: oracle.prism_gravity(coords, prisms, rho, f) for f in ("g_ee", "g_nn", "g_zz")}
    npt.assert_allclose(d["g_ee"] + d["g_nn"], -d["g_zz"], rtol=1e-7, atol=1e-9)


def test_null_prisms_and_disable_checks(oracle):
    e, n = np.meshgrid(np.linspace(-50, 50, 3), np.linspace(-50, 50, 3))
    coords = (e, n, np.zeros_like(e))
    prisms = [
        [-100, 100, -200, 200, -10e3, -5e3],
        [100, 200, 200, 300, -10e3, -4e3],
        [30, 30, -200, 200, -10e3, -5e3],
        [100, 200, 30, 30, -10e3, -5e3],
        [-100, 100, -200, 200, -10e3, -10e3],
    ]
    density = [2600, 0, 3000, 3100, 3200]
    npt.assert_allclose(
        oracle.prism_gravity(coords, prisms, density, "g_z"),
        oracle.prism_gravity(coords, [prisms[0]], [density[0]], "g_z"),
    )
    valid, invalid = [0, 10, 0, 10, -10, 0], [0, 10, 0, 10, 0, -10]
    with pytest.raises(ValueError, match="The bottom boundary can't be greater than the top one"):
        oracle.prism_gravity([0, 0, 0], invalid, 100, "potential")
    npt.assert_allclose(
        oracle.prism_gravity([0, 0, 0], invalid, 100, "potential", disable_checks=True),
        -oracle.prism_gravity([0, 0, 0], valid, 100, "potential"),
    )


def _vertices(p):
    return tuple(c.ravel() for c in np.meshgrid(p[:2], p[2:4], p[4:6]))


@pytest.mark.parametrize("field", ["g_ee", "g_nn", "g_zz", "g_en", "g_ez", "g_nz"])
def test_singular_vertices_warn_and_nan(oracle, field):
    """test/test_prism.py:380-400, plus NaN values at singular points."""
    prism = np.array([-10.3, 5.4, 8.6, 14.3, -30.3, 2.4])
    e, n, u = _vertices(prism)
    for i in range(e.size):
        with pytest.warns(UserWarning, match="Found observation point"):
            v = oracle.prism_gravity((e[i], n[i], u[i]), prism, [2900.0], field)
        assert np.isnan(v)


def test_singular_edges(oracle):
    """test/test_prism.py:402-502: edge midpoints of each direction."""
    prism = np.array([-10.3, 5.4, 8.6, 14.3, -30.3, 2.4])
    ec = (prism[0] + prism[1]) / 2
    nc = (prism[2] + prism[3]) / 2
    uc = (prism[4] + prism[5]) / 2
    n, u = (c.ravel() for c in np.meshgrid(prism[2:4], prism[4:6]))
    easting_edges = (np.full_like(n, ec), n, u)
    e, u = (c.ravel() for c in np.meshgrid(prism[0:2], prism[4:6]))
    northing_edges = (e, np.full_like(e, nc), u)
    e, n = (c.ravel() for c in np.meshgrid(prism[0:2], prism[2:4]))
    upward_edges = (e, n, np.full_like(e, uc))
    cases = {
        "easting": (easting_edges, ("g_nn", "g_zz", "g_nz"), ("g_ee", "g_en", "g_ez")),
        "northing": (northing_edges, ("g_ee", "g_zz", "g_ez"), ("g_nn", "g_en", "g_nz")),
        "upward": (upward_edges, ("g_ee", "g_nn", "g_en"), ("g_zz", "g_ez", "g_nz")),
    }
    for _, (pts, singular, regular) in cases.items():
        for i in range(pts[0].size):
            p = (pts[0][i], pts[1][i], pts[2][i])
            for f in singular:
                with pytest.warns(UserWarning, match="Found observation point"):
                    assert np.isnan(oracle.prism_gravity(p, prism, [2900.0], f))
            for f in regular:
                with warnings.catch_warnings():
                    warnings.simplefilter("error")
                    assert np.isfinite(oracle.prism_gravity(p, prism, [2900.0], f))
    # potential and accelerations are finite everywhere, vertices included
    e, n, u = _vertices(prism)
    for f in ("potential", "g_e", "g_n", "g_z"):
        assert np.all(np.isfinite(oracle.prism_gravity((e, n, u), prism, [2900.0], f)))


def test_against_mpmath(oracle):
    mp_check = pytest.importorskip("oracle.mp_check")
    rng = np.random.default_rng(5)
    for _ in range(6):
        w, s, b = rng.uniform(-500, 500, 3)
        prism = [w, w + rng.uniform(10, 300), s, s + rng.uniform(10, 300), b - 600,
                 b - 600 + rng.uniform(10, 300)]
        point = rng.uniform(-800, 800, 3)
        for f in FIELDS:
            ref = float(mp_check.prism_kernel(f, point, prism, 2000.0))
            val = oracle.prism_kernel(f, point, prism, 2000.0)
            npt.assert_allclose(val, ref, rtol=1e-9, err_msg=f)


def test_layer_oracle_matches_prism_list(oracle):
    g = np.load(os.path.join(GOLDEN, "oracle_small.npz"))
    e, n = g["layer_easting"], g["layer_northing"]
    ge, gn = np.meshgrid(e, n)
    he, hn = (e[1] - e[0]) / 2, (n[1] - n[0]) / 2
    prisms = np.column_stack(
        [ge.ravel() - he, ge.ravel() + he, gn.ravel() - hn, gn.ravel() + hn,
         g["layer_bottom"].ravel(), g["layer_top"].ravel()]
    )
    coords = (g["layer_obs_e"], g["layer_obs_n"], g["layer_obs_u"])
    for f in FIELDS:
        npt.assert_allclose(
            oracle.prism_gravity(coords, prisms, g["layer_density"].ravel(), f),
            g[f"layer_{f}"],
            rtol=1e-10,
            atol=1e-12 * np.max(np.abs(g[f"layer_{f}"])),
        )
