"""
The CUDA path against exact values: 50-digit evaluations of the closed form
(tests/golden/mp_truth.npz, written by tests/golden/make_mp_golden.py), so
the GPU machine needs no mpmath.  Every path a user can reach is checked: the
single-field kernels (prism_gravity), the fused all-field kernel
(prism_gravity_fields) and the layer kernels (the prism_layer accessor and
the fused layer launch).

Tolerances, against the exact value t of each output:

* near prisms (0.3 and 5 km from the prism centre), the points on face
  planes, edge lines and vertices, and the 64 x 64 sample of the 1e6-prism
  layer: |gpu - t| <= 1e-8 |t| + 1e-9 max|t| (the parity bar of the task);
  NaN exactly where the reference returns NaN;
* far single prisms (50 and 300 km, up to 6000 prism sizes away), where the
  closed form cancels: per distance class, the largest relative error of the
  GPU path is below the largest relative error of the reference's own
  algorithm evaluated in FP64 (the per-vertex oracle), i.e. the GPU result is
  at least as accurate as the reference itself there, and below 1e-4.
"""

import os
import warnings

import numpy as np
import numpy.testing as npt
import pytest

import harmonica_gb300 as hg

pytestmark = pytest.mark.gpu

FIXTURE = os.path.join(os.path.dirname(__file__), "golden", "mp_truth.npz")
FIELDS = hg.FIELDS
RTOL, ATOL_FRAC = 1e-8, 1e-9


@pytest.fixture(scope="module")
def truth():
    return np.load(FIXTURE)


def _bar(actual, exact, msg):
    actual, exact = np.asarray(actual), np.asarray(exact)
    npt.assert_array_equal(np.isnan(actual), np.isnan(exact), err_msg=msg)
    ok = np.isfinite(exact)
    atol = ATOL_FRAC * np.abs(exact[ok]).max()
    npt.assert_allclose(actual[ok], exact[ok], rtol=RTOL, atol=atol, err_msg=msg)


def _single(truth, field, fused):
    """Per point: (class km, value) of the single-prism cases on the GPU."""
    sp, sd = truth["single_prisms"], truth["single_density"]
    pts, which = truth["single_points"], truth["single_which"]
    out = np.empty(pts.shape[0])
    for k in range(sp.shape[0]):
        sel = which == k
        coords = tuple(pts[sel, c] for c in range(3))
        if fused:
            # all ten fields: one field alone would run the single-field kernel
            out[sel] = hg.prism_gravity_fields(coords, sp[k], [sd[k]], FIELDS)[field]
        else:
            out[sel] = hg.prism_gravity(coords, sp[k], [sd[k]], field=field)
    return out


@pytest.mark.parametrize("fused", [False, True], ids=["single-field", "fused"])
@pytest.mark.parametrize("field", FIELDS)
def test_single_prisms_near(gpu_lib, truth, field, fused):
    exact = truth[f"single_{field}"]
    near = truth["single_class"] <= 5.0
    got = _single(truth, field, fused)
    rel = np.abs(got[near] - exact[near]) / np.abs(exact[near])
    assert rel.max() <= RTOL, (field, rel.max())


@pytest.mark.parametrize("fused", [False, True], ids=["single-field", "fused"])
@pytest.mark.parametrize("field", FIELDS)
def test_single_prisms_far_at_least_as_accurate_as_the_reference(gpu_lib, oracle, truth, field,
                                                                 fused):
    exact = truth[f"single_{field}"]
    got = _single(truth, field, fused)
    sp, sd = truth["single_prisms"], truth["single_density"]
    pts, which, klass = truth["single_points"], truth["single_which"], truth["single_class"]
    ref = np.array([
        oracle.prism_gravity(tuple(pts[i:i + 1, c] for c in range(3)), sp[which[i]],
                             [sd[which[i]]], field)[0]
        for i in range(pts.shape[0])])
    for km in (50.0, 300.0):
        sel = klass == km
        ours = np.max(np.abs(got[sel] - exact[sel]) / np.abs(exact[sel]))
        theirs = np.max(np.abs(ref[sel] - exact[sel]) / np.abs(exact[sel]))
        assert ours <= max(theirs, RTOL) and ours <= 1e-4, (field, km, ours, theirs)


@pytest.mark.parametrize("field", FIELDS)
def test_faces_edges_and_vertices(gpu_lib, truth, field):
    pts = truth["faces_points"]
    coords = tuple(pts[:, c] for c in range(3))
    prism, rho = truth["faces_prism"], float(truth["faces_density"])
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")  # singular points of the tensor fields
        single = hg.prism_gravity(coords, prism, [rho], field=field)
        fused = hg.prism_gravity_fields(coords, prism, [rho], FIELDS)[field]
    _bar(single, truth[f"faces_{field}"], f"{field} single-field")
    _bar(fused, truth[f"faces_{field}"], f"{field} fused")


def test_layer_sample_every_path(gpu_lib, truth):
    """64 stations x the 8 x 8-prism block of the 1e6-prism layer, all ten
    fields, through the prism list (single-field and fused kernels) and the
    layer (accessor per field and the fused layer launch)."""
    from harmonica_gb300.layer import layer_forward

    pts = truth["layer_points"]
    coords = tuple(pts[:, c] for c in range(3))
    prisms, density = truth["layer_prisms"], truth["layer_density"]
    layer = hg.prism_layer((truth["layer_easting"], truth["layer_northing"]),
                           truth["layer_top"], truth["layer_bottom"],
                           properties={"density": density})
    npt.assert_array_equal(layer.prism_layer._to_prisms(), prisms)
    fused_list = hg.prism_gravity_fields(coords, prisms, density.ravel(), FIELDS)
    fused_layer = layer_forward(coords, truth["layer_easting"], truth["layer_northing"],
                                truth["layer_bottom"], truth["layer_top"], density, 0x3FF, 0.0)
    for code, field in enumerate(FIELDS):
        exact = truth[f"layer_{field}"]
        _bar(hg.prism_gravity(coords, prisms, density.ravel(), field=field), exact,
             f"{field} list single-field")
        _bar(fused_list[field], exact, f"{field} list fused")
        _bar(layer.prism_layer.gravity(coords, field=field), exact, f"{field} layer accessor")
        _bar(fused_layer[code], exact, f"{field} layer fused")
