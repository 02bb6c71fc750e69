"""Host logic of batching on CPU: the autotuner's problem-set signature and
its cache file (a corrupt or missing cache reads as empty)."""

import numpy as np

from harmonica_gb300.batch import _load_cache, signature


def _problem(n_obs, n_prisms, field):
    return {"coordinates": (np.zeros(n_obs), np.zeros(n_obs), np.zeros(n_obs)),
            "prisms": np.zeros((n_prisms, 6)), "density": np.zeros(n_prisms), "field": field}


def test_signature_counts_pairs_and_fields():
    probs = [_problem(1000, 2000, "g_z"), _problem(10, 30, "g_zz"), _problem(5, 5, "g_z")]
    pairs = 1000 * 2000 + 10 * 30 + 5 * 5
    assert signature(probs) == f"n3-p{int(np.log2(pairs))}-g_z+g_zz"
    # the same mix with the same order of magnitude of work shares a key
    probs2 = [_problem(1000, 2001, "g_z"), _problem(10, 30, "g_zz"), _problem(5, 5, "g_z")]
    assert signature(probs2) == signature(probs)
    assert signature([]) == "n0-p0-"


def test_cache_missing_or_corrupt_reads_empty(tmp_path):
    assert _load_cache(str(tmp_path / "missing.json")) == {}
    bad = tmp_path / "bad.json"
    bad.write_text("{not json")
    assert _load_cache(str(bad)) == {}
    good = tmp_path / "good.json"
    good.write_text('{"k": {"chunk_prisms": 2048, "n_ctas": 304}}')
    assert _load_cache(str(good))["k"]["n_ctas"] == 304
