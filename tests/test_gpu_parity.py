"""
Parity of the CUDA path (through the C ABI) with the CPU oracle, and the
behavioural tests of harmonica's own suite run on the GPU.

Tolerance (FP64 forward): |gpu - oracle| <= 1e-8 |oracle| + 1e-9 max|oracle|
per output array, unless a test states otherwise.
"""

import json
import os
import warnings

import numpy as np
import numpy.testing as npt
import pytest

import harmonica_gb300 as hg

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
FIELDS = hg.FIELDS
RTOL = 1e-8
ATOL_FRAC = 1e-9


def assert_parity(actual, expected, rtol=RTOL, atol_frac=ATOL_FRAC, msg="", floor=0.0):
    """floor: absolute tolerance for arrays that vanish by symmetry (rounding noise only)."""
    expected = np.asarray(expected)
    finite = np.isfinite(expected)
    atol = atol_frac * (np.max(np.abs(expected[finite])) if finite.any() else 0.0)
    atol = max(atol, floor)
    npt.assert_allclose(actual, expected, rtol=rtol, atol=atol, err_msg=msg)


def random_problem(seed, n_prisms, n_obs, spread=5e3):
    rng = np.random.default_rng(seed)
    west = rng.uniform(-spread, spread * 0.8, n_prisms)
    south = rng.uniform(-spread, spread * 0.8, n_prisms)
    bottom = rng.uniform(-3e3, -200, n_prisms)
    prisms = np.column_stack(
        [
            west,
            west + rng.uniform(20, 1500, n_prisms),
            south,
            south + rng.uniform(20, 1500, n_prisms),
            bottom,
            bottom + rng.uniform(20, 1500, n_prisms),
        ]
    )
    density = rng.uniform(-600, 600, n_prisms)
    coords = (
        rng.uniform(-1.2 * spread, 1.2 * spread, n_obs),
        rng.uniform(-1.2 * spread, 1.2 * spread, n_obs),
        rng.uniform(-500, 800, n_obs),  # some points inside/below prisms
    )
    return coords, prisms, density


def test_reference_doctest_vectors(gpu_lib):
    gold = json.load(open(os.path.join(GOLDEN, "reference_doctests.json")))
    for case in ("single_prism", "two_prisms"):
        c = gold[case]
        gz = hg.prism_gravity(gold["coordinates"], c["prisms"], c["density"], field="g_z")
        npt.assert_allclose(np.round(gz, 5), c["g_z"], rtol=0, atol=0)


@pytest.mark.parametrize("field", FIELDS)
def test_against_golden_choclo_fixture(gpu_lib, field):
    """TestAgainstChoclo inputs (test/test_prism.py:161-244) vs oracle fixture."""
    g = np.load(os.path.join(GOLDEN, "oracle_small.npz"))
    coords = (g["choclo_e"], g["choclo_n"], g["choclo_u"])
    result = hg.prism_gravity(coords, g["choclo_prisms"], g["choclo_density"], field=field)
    assert_parity(result, g[f"choclo_{field}"], msg=field)


@pytest.mark.parametrize("field", FIELDS)
def test_random_prisms_against_oracle(gpu_lib, oracle, field):
    coords, prisms, density = random_problem(1, 400, 300)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        ref = oracle.prism_gravity(coords, prisms, density, field)
        res = hg.prism_gravity(coords, prisms, density, field=field)
    assert_parity(res, ref, msg=field)


def test_extreme_aspect_ratios_against_oracle(gpu_lib, oracle):
    """Needles, plates and slabs (extents from 0.5 m to 2 km in one prism),
    every field alone and the ten fused, against the oracle."""
    rng = np.random.default_rng(21)
    shapes = [(0.5, 500.0, 50.0), (500.0, 0.5, 50.0), (500.0, 50.0, 0.5), (2000.0, 2000.0, 1.0),
              (1.0, 1.0, 2000.0), (0.5, 2000.0, 0.5)]
    prisms = []
    for dx, dy, dz in shapes:
        for _ in range(40):
            w, s = rng.uniform(-300, 300, 2)
            b = rng.uniform(-600, -10)
            prisms.append([w, w + dx, s, s + dy, b, b + dz])
    prisms = np.array(prisms)
    rho = rng.uniform(-3000, 3000, len(prisms))
    n = 300
    coords = (rng.uniform(-3e3, 3e3, n), rng.uniform(-3e3, 3e3, n), rng.uniform(-700, 300, n))
    fused = hg.prism_gravity_fields(coords, prisms, rho, FIELDS)
    for field in FIELDS:
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            ref = oracle.prism_gravity(coords, prisms, rho, field)
        assert_parity(hg.prism_gravity(coords, prisms, rho, field=field), ref, msg=field)
        assert_parity(fused[field], ref, msg="fused " + field)


@pytest.mark.parametrize("field", FIELDS)
def test_progress_bar(gpu_lib, capsys, field):
    """test/test_prism.py:367-377: results with and without the progress bar
    match; here the bar is a line on stderr, printed per chunk of points."""
    coords, prisms, density = random_problem(4, 60, 250)
    with_bar = hg.prism_gravity(coords, prisms, density, field=field, progressbar=True)
    err = capsys.readouterr().err
    assert "250/250 points" in err and "(100.0%)" in err
    without = hg.prism_gravity(coords, prisms, density, field=field, progressbar=False)
    assert capsys.readouterr().err == ""
    npt.assert_allclose(with_bar, without, rtol=1e-12, atol=1e-13 * np.max(np.abs(without)))


def test_fused_all_fields_match_single(gpu_lib):
    coords, prisms, density = random_problem(2, 257, 190)
    fused = hg.prism_gravity_fields(coords, prisms, density, FIELDS)
    for f in FIELDS:
        single = hg.prism_gravity(coords, prisms, density, field=f)
        npt.assert_allclose(fused[f], single, rtol=1e-10, atol=1e-11 * np.max(np.abs(single)))


def test_many_chunks_and_ragged_sizes(gpu_lib, oracle):
    """Sizes not multiples of the tiles, and the ways the launch splits the
    work: one point tile over many prism chunks (few points, many prisms),
    many point tiles and one chunk (many points, few prisms), and both."""
    for n_obs, n_prisms in ((1, 1), (3, 129), (7, 5000), (129, 1), (300, 3001), (1000, 700),
                            (2000, 20000), (64, 100000), (20000, 130)):
        coords, prisms, density = random_problem(n_obs + n_prisms, n_prisms, n_obs)
        ref = oracle.prism_gravity(coords, prisms, density, "g_z")
        res = hg.prism_gravity(coords, prisms, density, field="g_z")
        assert_parity(res, ref, msg=f"{n_obs}x{n_prisms}")


def test_empty_inputs(gpu_lib):
    res = hg.prism_gravity((np.zeros(0), np.zeros(0), np.zeros(0)), [0, 1, 0, 1, -1, 0], 1.0,
                           field="g_z")
    assert res.shape == (0,)
    # only null prisms -> zeros (gravity.py:452-486 discards them)
    res = hg.prism_gravity(([0.0, 5.0], [0.0, 1.0], [1.0, 1.0]), [[0, 0, 0, 1, -1, 0]], [10.0],
                           field="g_z")
    npt.assert_array_equal(res, np.zeros(2))


def test_output_shape_and_dtype(gpu_lib):
    e, n = np.meshgrid(np.linspace(-100, 100, 4), np.linspace(-50, 50, 3))
    res = hg.prism_gravity((e, n, 10.0), [-20, 20, -20, 20, -50, -10], 2000, field="g_z",
                           dtype="float32")
    assert res.shape == (3, 4) and res.dtype == np.float32


def test_infinite_slab(gpu_lib):
    """test/test_prism.py:269-297"""
    height, thickness, density = 1.5, 10.5, 2670
    sizes = np.logspace(3, 9, 7)
    results = np.array(
        [
            hg.prism_gravity(
                (0, 0, height), [-s / 2, s / 2, -s / 2, s / 2, height - thickness, height],
                density, field="g_z",
            )
            for s in sizes
        ]
    )
    analytical = 1e5 * 2 * np.pi * 6.6743e-11 * density * thickness
    errors = np.abs(analytical - results)
    assert (errors[1:] < errors[:-1]).all()
    npt.assert_allclose(analytical, results[-1], rtol=1e-7)


def test_laplace(gpu_lib):
    """test/test_prism.py:247-266"""
    e, n = np.meshgrid(np.linspace(-10e3, 10e3, 10), np.linspace(-10e3, 10e3, 10))
    coords = (e, n, np.full_like(e, 300.0))
    prisms = [[1e3, 7e3, -5e3, 2e3, -1e3, -500], [-4e3, 1e3, 4e3, 10e3, -2e3, 200]]
    rho = [2670.0, 2900.0]
    d = {f: hg.prism_gravity(coords, prisms, rho, field=f) for f in ("g_ee", "g_nn", "g_zz")}
    npt.assert_allclose(d["g_ee"] + d["g_nn"], -d["g_zz"], rtol=1e-7, atol=1e-9)


def test_null_prisms_and_disable_checks(gpu_lib):
    """test/test_prism.py:115-158"""
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
        hg.prism_gravity(coords, prisms, density, field="g_z"),
        hg.prism_gravity(coords, [prisms[0]], [density[0]], field="g_z"),
    )
    valid, invalid = [0, 10, 0, 10, -10, 0], [0, 10, 0, 10, 0, -10]
    npt.assert_allclose(
        hg.prism_gravity([0, 0, 0], invalid, 100, field="potential", disable_checks=True),
        -hg.prism_gravity([0, 0, 0], valid, 100, field="potential"),
    )


def _vertices(p):
    return tuple(c.ravel() for c in np.meshgrid(p[:2], p[2:4], p[4:6]))


@pytest.mark.parametrize("field", ["g_ee", "g_nn", "g_zz", "g_en", "g_ez", "g_nz"])
def test_singular_vertices(gpu_lib, field):
    """test/test_prism.py:380-400: warning, and NaN values (gravity.py:151)."""
    prism = np.array([-10.3, 5.4, 8.6, 14.3, -30.3, 2.4])
    e, n, u = _vertices(prism)
    for i in range(e.size):
        with pytest.warns(UserWarning, match="Found observation point"):
            v = hg.prism_gravity((e[i], n[i], u[i]), prism, [2900.0], field=field)
        assert np.isnan(v)
    # no warning with disable_checks, still NaN
    with warnings.catch_warnings():
        warnings.simplefilter("error")
        v = hg.prism_gravity((e[0], n[0], u[0]), prism, [2900.0], field=field,
                             disable_checks=True)
    assert np.isnan(v)


def test_singular_edges_and_regular_neighbours(gpu_lib, oracle):
    """test/test_prism.py:402-502 and finiteness of the other components."""
    prism = np.array([-10.3, 5.4, 8.6, 14.3, -30.3, 2.4])
    ec, nc, uc = (prism[0] + prism[1]) / 2, (prism[2] + prism[3]) / 2, (prism[4] + prism[5]) / 2
    n, u = (c.ravel() for c in np.meshgrid(prism[2:4], prism[4:6]))
    e_edges = (np.full_like(n, ec), n, u)
    e, u = (c.ravel() for c in np.meshgrid(prism[0:2], prism[4:6]))
    n_edges = (e, np.full_like(e, nc), u)
    e, n = (c.ravel() for c in np.meshgrid(prism[0:2], prism[2:4]))
    u_edges = (e, n, np.full_like(e, uc))
    cases = [
        (e_edges, ("g_nn", "g_zz", "g_nz"), ("g_ee", "g_en", "g_ez")),
        (n_edges, ("g_ee", "g_zz", "g_ez"), ("g_nn", "g_en", "g_nz")),
        (u_edges, ("g_ee", "g_nn", "g_en"), ("g_zz", "g_ez", "g_nz")),
    ]
    for pts, singular, regular in cases:
        for f in singular:
            with pytest.warns(UserWarning, match="Found observation point"):
                v = hg.prism_gravity(pts, prism, [2900.0], field=f)
            assert np.all(np.isnan(v))
        for f in regular + ("potential", "g_e", "g_n", "g_z"):
            with warnings.catch_warnings():
                warnings.simplefilter("error")
                v = hg.prism_gravity(pts, prism, [2900.0], field=f)
            # some components vanish by symmetry on these points: 1e-12 floor
            assert_parity(v, oracle.prism_gravity(pts, prism, [2900.0], f), msg=f, floor=1e-12)


def test_points_on_faces_and_edge_extensions(gpu_lib, oracle):
    """Face planes (outside limit of diagonal tensors) and extensions of edges."""
    prism = np.array([-10.0, 20.0, -5.0, 15.0, -40.0, -10.0])
    pts = []
    for e in (-10.0, 20.0, 5.0, -30.0, 40.0):
        for n in (-5.0, 15.0, 3.0, -25.0, 35.0):
            for u in (-40.0, -10.0, -20.0, 5.0, -60.0):
                pts.append((e, n, u))
    pts = np.array(pts)
    coords = (pts[:, 0], pts[:, 1], pts[:, 2])
    for f in FIELDS:
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            ref = oracle.prism_gravity(coords, prism, [1000.0], f)
            res = hg.prism_gravity(coords, prism, [1000.0], field=f)
        npt.assert_array_equal(np.isnan(res), np.isnan(ref), err_msg=f)
        ok = np.isfinite(ref)
        assert_parity(res[ok], ref[ok], msg=f)


def test_determinism(gpu_lib):
    coords, prisms, density = random_problem(3, 2000, 50)
    a = hg.prism_gravity(coords, prisms, density, field="g_z")
    b = hg.prism_gravity(coords, prisms, density, field="g_z")
    npt.assert_array_equal(a, b)


def test_float32_dtype_at_least_as_accurate_as_the_reference(gpu_lib, oracle):
    """dtype="float32": the reference accumulates in the user's dtype
    (gravity.py:201, :524-537: out[i] += kernel, stored as float32 after every
    prism); here the sum runs in FP64 and is rounded to float32 once.  The
    result is never further from the exact sum than the reference's float32
    accumulation (restated here around the oracle's per-pair kernels), and is
    the FP64 result correctly rounded to float32."""
    coords, prisms, density = random_problem(21, 3000, 64)
    ours = hg.prism_gravity(coords, prisms, density, field="g_z", dtype="float32")
    assert ours.dtype == np.float32
    exact = hg.prism_gravity(coords, prisms, density, field="g_z")
    npt.assert_array_equal(ours, exact.astype(np.float32))
    # the reference's float32 accumulation of the raw (SI, upward) kernels,
    # prism after prism in its order, then its sign flip and mGal scaling in
    # float32; the per-pair raw values come from the oracle (g_z = -1e5 raw)
    raw = np.column_stack([oracle.prism_gravity(coords, p, [d], "g_z") / -1e5
                           for p, d in zip(prisms, density)])
    acc = np.zeros(raw.shape[0], dtype=np.float32)
    for j in range(raw.shape[1]):
        acc = (acc.astype(np.float64) + raw[:, j]).astype(np.float32)
    ref32 = (acc * np.float32(-1)) * np.float32(1e5)
    exact_sum = -1e5 * raw.sum(axis=1)
    assert np.all(np.abs(ours - exact_sum) <= np.abs(ref32 - exact_sum)
                  + np.spacing(np.abs(ours)))


def test_pairs_near_a_plane_of_a_distant_prism(gpu_lib, oracle):
    """Pairs with one bound far smaller than the largest (a station a few mm
    to a few m from the plane of a face of a prism kilometres away): the
    potential and the fused all-field forward run as an edge-log launch and
    a face launch, which send these pairs whole to the FP64 path (when a
    bound is below 2^-14 of the pair's scale) in the first and skip them in
    the second.  Against the oracle at the parity bar, single-field and
    fused, on both sides of the 2^-14 threshold."""
    rng = np.random.default_rng(12)
    prisms, coords = [], ([], [], [])
    for k in range(40):
        west = rng.uniform(2e3, 2e4) * rng.choice([-1, 1])
        south = rng.uniform(-5e3, 5e3)
        bottom = -rng.uniform(2e3, 8e3)
        p = [west, west + rng.uniform(100, 800), south, south + rng.uniform(100, 800),
             bottom, bottom + rng.uniform(100, 2000)]
        prisms.append(p)
    prisms = np.array(prisms)
    density = rng.uniform(1000, 3000, prisms.shape[0])
    # stations offset from the planes x = west, y = south, z = top of every
    # prism by 1e-3 .. 10 m (log-uniform), elsewhere at random
    for p in prisms:
        for axis in range(3):
            for off in np.exp(rng.uniform(np.log(1e-3), np.log(10.0), 3)):
                pt = [rng.uniform(-3e4, 3e4), rng.uniform(-3e4, 3e4), rng.uniform(10, 500)]
                plane = (p[0], p[2], p[5])[axis]
                pt[axis] = plane + off * rng.choice([-1, 1])
                for c in range(3):
                    coords[c].append(pt[c])
    coords = tuple(np.array(c) for c in coords)
    fused = hg.prism_gravity_fields(coords, prisms, density, FIELDS)
    for f in FIELDS:
        ref = oracle.prism_gravity(coords, prisms, density, f)
        assert_parity(hg.prism_gravity(coords, prisms, density, field=f), ref, msg=f)
        assert_parity(fused[f], ref, msg=f"fused {f}")
