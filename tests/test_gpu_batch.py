"""
Batched persistent launch (hg_batch_*): results equal the single-problem
drop-in, are bitwise the same alone and in a mixed batch (fixed chunking),
survive CUDA-graph capture/replay, and cover every field, empty problems and
singular flags.  Tolerance vs the oracle: 1e-8 rel + 1e-9 max|oracle| abs.
"""

import warnings

import numpy as np
import numpy.testing as npt
import pytest

import harmonica_gb300 as hg
from harmonica_gb300 import synthetic

pytestmark = pytest.mark.gpu


def small_set(seed=0, n=12):
    probs = synthetic.batched_problems(n, seed=seed, scale=0.02)
    fields = hg.FIELDS
    for k, p in enumerate(probs):
        p["field"] = fields[k % len(fields)]
    return probs


def test_batch_matches_single_and_oracle(gpu_lib, oracle):
    probs = small_set()
    res = hg.prism_gravity_batch(probs, disable_checks=True)
    for p, r in zip(probs, res):
        single = hg.prism_gravity(p["coordinates"], p["prisms"], p["density"], field=p["field"],
                                  disable_checks=True)
        npt.assert_allclose(r, single, rtol=1e-10, atol=1e-11 * np.abs(single).max())
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            ref = oracle.prism_gravity(p["coordinates"], p["prisms"], p["density"], p["field"],
                                       disable_checks=True)
        npt.assert_allclose(r, ref, rtol=1e-8, atol=1e-9 * np.abs(ref).max())


def test_alone_and_in_mix_bitwise(gpu_lib):
    probs = small_set(seed=1, n=10)
    mix = hg.PrismBatch(probs, chunk_prisms=256)
    mix.run()
    mixed = mix.results()
    mix.close()
    for k in (0, 3, 7):
        alone = hg.PrismBatch([probs[k]], chunk_prisms=256)
        alone.run()
        npt.assert_array_equal(alone.results()[0], mixed[k])
        alone.close()


def test_graph_capture_and_replay(gpu_lib):
    import torch

    probs = small_set(seed=2, n=6)
    b = hg.PrismBatch(probs, chunk_prisms=512)
    b.capture()
    b.replay()
    first = b.results()
    # change one input in place: the replay recomputes from current buffers
    b._keep[3].mul_(2.0)  # problem 0's prism SoA (densities doubled, geometry doubled too)
    b.replay()
    second = b.results()
    assert not np.allclose(first[0], second[0])
    for a, c in zip(first[1:], second[1:]):
        npt.assert_array_equal(a, c)
    b._keep[3].mul_(0.5)
    b.replay()
    npt.assert_array_equal(b.results()[0], first[0])
    torch.cuda.synchronize()
    b.close()


def test_empty_problems_and_flags(gpu_lib):
    prism = np.array([[-10.3, 5.4, 8.6, 14.3, -30.3, 2.4]])
    probs = [
        dict(coordinates=(np.zeros(0), np.zeros(0), np.zeros(0)), prisms=prism,
             density=[1.0], field="g_z"),
        dict(coordinates=([0.0, 1.0], [0.0, 1.0], [1.0, 1.0]), prisms=np.zeros((0, 6)),
             density=np.zeros(0), field="g_z"),
        dict(coordinates=([-10.3], [8.6], [2.4]), prisms=prism, density=[2900.0],
             field="g_zz"),
        dict(coordinates=([100.0], [100.0], [100.0]), prisms=prism, density=[2900.0],
             field="g_zz"),
    ]
    b = hg.PrismBatch(probs, check_singular=True)
    b.run()
    res = b.results()
    assert res[0].shape == (0,)
    npt.assert_array_equal(res[1], np.zeros(2))
    assert np.isnan(res[2][0]) and np.isfinite(res[3][0])
    npt.assert_array_equal(b.singular(), [False, False, True, False])
    b.close()
    with pytest.warns(UserWarning, match="Found observation point"):
        hg.prism_gravity_batch(probs)


def test_autotune_picks_a_shape_per_field_and_caches_it(gpu_lib, tmp_path):
    probs = small_set(seed=3, n=8)
    kw = dict(chunks=(256, 1024), points_per_cta=(64, 128), cta_multipliers=(1,), repeats=1,
              cache=str(tmp_path / "tune.json"))
    choice = hg.autotune(probs, **kw)
    fields = {p["field"] for p in probs}
    assert set(choice["shapes"]) == fields
    for shape in choice["shapes"].values():
        assert shape["chunk_prisms"] in (256, 1024) and shape["points_per_cta"] in (64, 128)
        assert shape["gain"] > 0
    assert len(choice["candidates"]) == 4 * len(fields)
    assert hg.autotune(probs, **kw) == choice  # from the cache


def test_every_shape_gives_the_same_results(gpu_lib, oracle):
    """64 and 128 points per CTA (prism tiles of the same size) and several
    chunks give the same results, within rounding, as the oracle."""
    probs = small_set(seed=5, n=10)
    ref = [oracle.prism_gravity(p["coordinates"], p["prisms"], p["density"], p["field"],
                                disable_checks=True) for p in probs]
    for ppc in (64, 128):
        for chunk in (64, 320, 4096):
            shapes = {f: {"chunk_prisms": chunk, "points_per_cta": ppc, "n_ctas": 0}
                      for f in hg.FIELDS}
            res = hg.prism_gravity_batch(probs, disable_checks=True, shapes=shapes)
            for r, e in zip(res, ref):
                npt.assert_allclose(r, e, rtol=1e-8, atol=1e-9 * np.abs(e).max(),
                                    err_msg=f"{ppc} points per CTA, chunk {chunk}")


def test_batched_workload_full_size_against_oracle(gpu_lib, oracle):
    """The batched workload at full size (256 problems of 1e3-2e5 prisms and
    1e3-5e4 stations, g_z and g_zz): every 31st problem (both fields) against
    the oracle on 48 of its stations (strided) and all of its prisms."""
    probs = synthetic.batched_problems(256, seed=4)
    res = hg.prism_gravity_batch(probs, disable_checks=True)
    for k in range(0, 256, 31):
        p = probs[k]
        n = p["coordinates"][0].size
        idx = np.linspace(0, n - 1, min(48, n)).astype(int)
        sub = tuple(np.ascontiguousarray(c[idx]) for c in p["coordinates"])
        ref = oracle.prism_gravity(sub, p["prisms"], p["density"], p["field"],
                                   disable_checks=True)
        npt.assert_allclose(res[k][idx], ref, rtol=1e-8, atol=1e-9 * np.abs(ref).max(),
                            err_msg=f"problem {k} ({p['field']})")
