"""
Serving loop with continuous batching (PrismServer): results equal the
drop-in, each result is bitwise the same alone and in a mix of concurrent
requests, admission respects the memory budget, resident layers are reused
and evicted, empty requests complete.  Tolerance vs the drop-in: 1e-12
relative (different chunking of the same FP64 sums).
"""

import concurrent.futures as cf

import numpy as np
import numpy.testing as npt
import pytest

import harmonica_gb300 as hg
from harmonica_gb300 import synthetic
from harmonica_gb300.serve import PrismServer

pytestmark = pytest.mark.gpu


def _requests(seed, n, scale=0.01):
    probs = synthetic.batched_problems(n, seed=seed, scale=scale)
    fields = ("g_z", "potential", "g_zz")
    for k, p in enumerate(probs):
        p["field"] = fields[k % 3]
    return probs


def test_results_match_drop_in(gpu_lib):
    probs = _requests(20, 9)
    # 5.4e5 pairs in all, work items of at most 128 x 512 pairs: many rounds
    srv = PrismServer(round_pairs=1e5)
    futs = [srv.submit(p["coordinates"], p["field"], prisms=p["prisms"], density=p["density"])
            for p in probs]
    res = [f.result(timeout=120) for f in futs]
    srv.close()
    for p, r in zip(probs, res):
        ref = hg.prism_gravity(p["coordinates"], p["prisms"], p["density"], field=p["field"])
        npt.assert_allclose(r, ref, rtol=1e-10, atol=1e-11 * np.abs(ref).max())
    st = srv.stats()
    assert st["completed"] == len(probs) and st["rounds"] > 1 and "p99_ms" in st


def test_alone_and_in_mix_bitwise(gpu_lib):
    probs = _requests(21, 12)
    target = probs[5]
    alone = PrismServer(round_pairs=1e6)
    ra = alone.submit(target["coordinates"], target["field"], prisms=target["prisms"],
                      density=target["density"]).result(timeout=120)
    alone.close()
    mix = PrismServer(round_pairs=1e6)
    futs = []
    for k, p in enumerate(probs):
        futs.append(mix.submit(p["coordinates"], p["field"], prisms=p["prisms"],
                               density=p["density"]))
    rm = futs[5].result(timeout=120)
    cf.wait(futs, timeout=120)
    mix.close()
    npt.assert_array_equal(ra, rm)


def test_resident_layer_and_admission_budget(gpu_lib):
    L = synthetic.layer_topography_1e6(n_side=40, n_stations_side=12)
    prisms, density = synthetic.layer_to_prisms(L)
    srv = PrismServer(memory_budget=3e6, round_pairs=5e5)
    layer_bytes = srv.register_layer("topo", prisms, density)
    assert layer_bytes == 7 * prisms.shape[0] * 8
    coords = L["coordinates"]
    futs = [srv.submit(tuple(c[k::4] for c in coords), "g_z", layer="topo") for k in range(4)]
    res = [f.result(timeout=120) for f in futs]
    ref = hg.prism_gravity(coords, prisms, density, field="g_z")
    for k, r in enumerate(res):
        npt.assert_allclose(r, ref[k::4], rtol=1e-10, atol=1e-11 * np.abs(ref).max())
    # a request that can never fit is rejected, the server keeps going
    big = (np.zeros(200_000), np.zeros(200_000), np.ones(200_000))
    with pytest.raises(MemoryError):
        srv.submit(big, "g_z", layer="topo").result(timeout=60)
    assert srv.submit(tuple(c[:5] for c in coords), "g_z", layer="topo").result(60).shape == (5,)
    srv.close()
    assert srv.used == pytest.approx(layer_bytes)


def test_empty_request_and_unknown_layer(gpu_lib):
    srv = PrismServer()
    r = srv.submit((np.zeros(3), np.zeros(3), np.ones(3)), "g_z", prisms=np.zeros((0, 6)),
                   density=np.zeros(0)).result(timeout=60)
    npt.assert_array_equal(r, np.zeros(3))
    with pytest.raises(KeyError):
        srv.submit((np.zeros(3), np.zeros(3), np.ones(3)), "g_z", layer="nope").result(60)
    srv.close()


def test_serving_stream_with_full_size_models(gpu_lib, oracle):
    """The first 12 requests of the serving workload with their full prism
    models (1e3-1e6 prisms; the resident share served from registered
    layers), station counts capped at 4000 to keep the test short.  Every
    served result equals the drop-in within 1e-10 (same FP64 sums, other
    chunking) and the CPU oracle on 16 strided stations within 1e-8."""
    models = synthetic.serving_models()
    stream = synthetic.serving_stream(seconds=0.5)[:12]
    srv = PrismServer(round_pairs=1.6e9)
    for k in sorted({r["model"] for r in stream if r["resident"]}):
        prisms, density, _ = models[k]
        srv.register_layer(f"model{k}", prisms, density)
    futs, inputs = [], []
    for req in stream:
        prisms, density, side = models[req["model"]]
        coords = synthetic.serving_request_coordinates(
            dict(req, n_stations=min(req["n_stations"], 4000)), side)
        if req["resident"]:
            futs.append(srv.submit(coords, req["field"], layer=f"model{req['model']}"))
        else:
            futs.append(srv.submit(coords, req["field"], prisms=prisms, density=density))
        inputs.append((coords, prisms, density, req["field"]))
    results = [f.result(timeout=300) for f in futs]
    srv.close()
    assert max(p.shape[0] for _, p, _, _ in inputs) > 1e5  # the large models are in
    for (coords, prisms, density, field), got in zip(inputs, results):
        ref = hg.prism_gravity(coords, prisms, density, field=field)
        npt.assert_allclose(got, ref, rtol=1e-10, atol=1e-11 * np.abs(ref).max())
        idx = np.linspace(0, coords[0].size - 1, 16).astype(int)
        truth = oracle.prism_gravity(tuple(c[idx] for c in coords), prisms, density, field)
        npt.assert_allclose(got[idx], truth, rtol=1e-8, atol=1e-9 * np.abs(truth).max())
