"""The reference arm of bench.py (the CPU path of the reference, timed on the
host) prints one JSON line with the keys the benchmark contract asks for;
it needs no GPU, so it runs here on a sample of two stations."""

import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_json_line():
    run = subprocess.run(
        [sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
         "--warmup", "0", "--cpu-sample-stations", "2"],
        capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert run.returncode == 0, run.stderr[-2000:]
    lines = [ln for ln in run.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference"
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
                "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config"):
        assert key in line, key
    assert line["metric"].startswith("FP64 g_z prism·station pairs/s, served vs plain")
    assert line["unit"] == "pairs/s"
    assert line["value"] > 0 and line["higher_is_better"] is True
    assert line["cpu_baseline"]["kind"] in ("port", "reference")
    assert line["cpu_baseline"]["cores"] >= 1 and line["cpu_baseline"]["value"] == line["value"]
    assert line["e2e"] == {"value": line["value"], "unit": "pairs/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    assert "workload" in line["config"]


def test_kernel_counts_match_the_kernel_sources():
    """The ncu counts that bench.py turns into the roofline fraction are keyed
    by a hash of the kernel sources; when the sources change without a new
    capture, the bench reports the counts as stale instead of using them."""
    sys.path.insert(0, ROOT)
    import bench

    sha = bench.kernel_sources_sha()
    assert len(sha) == 16
    counts = bench.KERNEL_COUNTS
    if counts["sources_sha"] is not None:
        for key in ("warp_inst_per_pair", "fp64_inst_per_pair", "capture"):
            assert counts[key] is not None, key
        assert counts["dram_bytes_default_step"] > 0
