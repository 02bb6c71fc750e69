"""
The edge/face formulation of the CUDA kernels (prism_math.cuh), compiled for
the host, against the per-vertex CPU oracle and 50-digit mpmath (no GPU).

This checks the regrouped closed form itself -- reflections, the
straddling-edge identity, face-plane limits, singular points -- on the CPU,
so the GPU tests only have to show that the device build computes the same.
"""

import ctypes
import os
import sys
import warnings

import numpy as np
import numpy.testing as npt
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "native"))

FIELDS = ("potential", "g_e", "g_n", "g_z", "g_ee", "g_nn", "g_zz", "g_en", "g_ez", "g_nz")


@pytest.fixture(scope="module")
def host():
    import build_host

    lib = ctypes.CDLL(build_host.build())
    dp = ctypes.POINTER(ctypes.c_double)
    lib.host_prism_gravity.argtypes = [
        ctypes.c_int, ctypes.c_int64, dp, dp, dp, ctypes.c_int64, dp, dp, dp, ctypes.c_int
    ]
    lib.host_prism_gravity.restype = None

    def run(coords, prisms, density, field, mode=0):
        cast = np.broadcast(*coords)
        e, n, u = (
            np.ascontiguousarray(np.broadcast_to(np.asarray(c, float), cast.shape)).ravel()
            for c in coords
        )
        p = np.ascontiguousarray(np.atleast_2d(np.asarray(prisms, float)))
        rho = np.ascontiguousarray(np.atleast_1d(np.asarray(density, float)))
        out = np.zeros(e.size)
        P = lambda a: a.ctypes.data_as(dp)  # noqa: E731
        lib.host_prism_gravity(FIELDS.index(field), e.size, P(e), P(n), P(u), p.shape[0], P(p),
                               P(rho), P(out), mode)
        return out.reshape(cast.shape)

    return run


def parity(a, b, rtol=1e-8, atol_frac=1e-9):
    b = np.asarray(b)
    fin = np.isfinite(b)
    atol = atol_frac * (np.abs(b[fin]).max() if fin.any() else 0)
    npt.assert_array_equal(np.isnan(a), np.isnan(b))
    npt.assert_allclose(np.asarray(a)[fin], b[fin], rtol=rtol, atol=atol)


MODES = {"lean": 0, "libm": 1, "fused": 2, "split": 3}


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("field", FIELDS)
def test_random_against_oracle(host, oracle, field, mode):
    rng = np.random.default_rng(3)
    m, n = 120, 150
    w = rng.uniform(-2e3, 2e3, m)
    s = rng.uniform(-2e3, 2e3, m)
    b = rng.uniform(-2e3, 200, m)
    prisms = np.column_stack([w, w + rng.uniform(5, 900, m), s, s + rng.uniform(5, 900, m), b,
                              b + rng.uniform(5, 900, m)])
    rho = rng.uniform(-500, 500, m)
    coords = (rng.uniform(-3e3, 3e3, n), rng.uniform(-3e3, 3e3, n), rng.uniform(-2e3, 1e3, n))
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        ref = oracle.prism_gravity(coords, prisms, rho, field)
    parity(host(coords, prisms, rho, field, MODES[mode]), ref)


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("field", FIELDS)
def test_special_points_against_oracle(host, oracle, field, mode):
    """Points on vertices, edges, faces, and on extensions of edges and faces."""
    prism = np.array([-10.0, 20.0, -5.0, 15.0, -40.0, -10.0])
    vals_e = (-10.0, 20.0, 5.0, -30.0, 40.0)
    vals_n = (-5.0, 15.0, 3.0, -25.0, 35.0)
    vals_u = (-40.0, -10.0, -20.0, 5.0, -60.0)
    pts = np.array([(e, n, u) for e in vals_e for n in vals_n for u in vals_u])
    coords = (pts[:, 0], pts[:, 1], pts[:, 2])
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        ref = oracle.prism_gravity(coords, prism, [1000.0], field)
    parity(host(coords, prism, [1000.0], field, MODES[mode]), ref)


@pytest.mark.parametrize("mode", ["lean", "fused", "split"])
@pytest.mark.parametrize("field", FIELDS)
def test_extreme_aspect_ratios_against_oracle(host, oracle, field, mode):
    """Needles, plates and slabs (extents from 0.5 m to 2 km in one prism):
    the regrouped combinations weight logs by bounds and extents of very
    different sizes (dP much smaller than p1, or the reverse), at points in
    and around the prisms and a few prism lengths away."""
    rng = np.random.default_rng(21)
    shapes = [(0.5, 500.0, 50.0), (500.0, 0.5, 50.0), (500.0, 50.0, 0.5), (2000.0, 2000.0, 1.0),
              (1.0, 1.0, 2000.0), (0.5, 2000.0, 0.5)]
    prisms = []
    for dx, dy, dz in shapes:
        for _ in range(4):
            w, s = rng.uniform(-300, 300, 2)
            b = rng.uniform(-600, -10)
            prisms.append([w, w + dx, s, s + dy, b, b + dz])
    prisms = np.array(prisms)
    rho = rng.uniform(-3000, 3000, len(prisms))
    n = 120
    coords = (rng.uniform(-3e3, 3e3, n), rng.uniform(-3e3, 3e3, n), rng.uniform(-700, 300, n))
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        ref = oracle.prism_gravity(coords, prisms, rho, field)
    parity(host(coords, prisms, rho, field, MODES[mode]), ref)


def test_distant_prism_accuracy_vs_mpmath(host, oracle):
    """At large distance the regrouped form is at least as accurate as the
    8-vertex sum (both measured against 50-digit arithmetic)."""
    mp_check = pytest.importorskip("oracle.mp_check")
    rng = np.random.default_rng(9)
    worse = []
    for _ in range(3):
        w, s = rng.uniform(-100, 100, 2)
        prism = [w, w + 50, s, s + 70, -2000, -1900]
        for dist in (5e3, 5e4, 5e5):
            pt = (dist * rng.uniform(0.5, 1), dist * rng.uniform(-1, 1), 100.0)
            for f in ("potential", "g_z", "g_e", "g_zz", "g_en"):
                ref = mp_check.prism_gravity(f, [pt], [prism], [2500.0])[0]
                ours = abs(host(pt, prism, [2500.0], f) - ref) / abs(ref)
                base = abs(oracle.prism_gravity(pt, prism, [2500.0], f) - ref) / abs(ref)
                if dist <= 5e3:
                    assert ours <= 1e-9, (f, dist, ours)
                worse.append((ours, base, f, dist))
    # never much worse than the per-vertex FP64 sum (typically 3-30x better)
    for ours, base, f, dist in worse:
        assert ours <= max(10 * base, 1e-9), (f, dist, ours, base)
    assert np.median([o for o, _, _, _ in worse]) < np.median([b for _, b, _, _ in worse])


@pytest.mark.parametrize("field", FIELDS)
def test_edge_and_face_parts_add_up_to_the_fused_pair(host, field):
    """The potential and fused all-field kernels run as an edge-log launch and
    a face launch whose sums add up to the fused pair (1e-12 relative to the
    field's largest value), near and far, including pairs that take the FP64
    path because a bound is tiny against the pair's scale."""
    rng = np.random.default_rng(9)
    m, n = 60, 80
    w = rng.uniform(-5e4, 5e4, m)
    s = rng.uniform(-5e4, 5e4, m)
    b = rng.uniform(-8e3, 0, m)
    prisms = np.column_stack([w, w + rng.uniform(50, 900, m), s, s + rng.uniform(50, 900, m), b,
                              b + rng.uniform(50, 3000, m)])
    rho = rng.uniform(1000, 3000, m)
    e, nn, u = (rng.uniform(-5e4, 5e4, n), rng.uniform(-5e4, 5e4, n), rng.uniform(10, 500, n))
    e[:10] = prisms[:10, 0] + 1e-3  # 1 mm from a face plane of a distant prism
    coords = (e, nn, u)
    fused = host(coords, prisms, rho, field, MODES["fused"])
    split = host(coords, prisms, rho, field, MODES["split"])
    npt.assert_allclose(split, fused, rtol=0, atol=1e-12 * np.abs(fused).max())
