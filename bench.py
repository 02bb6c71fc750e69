"""
Benchmark of the prism gravity forward model on one GB300: FP64 g_z
prism-station pairs/s of the plain drop-in, with the served and batched
forms of the same path beside it.

Workload of the headline (N=1): the 1e6-prism topography layer (1000 x 1000
prisms on a 200 m grid, 200 km square, Gaussian-sum tops, bottoms at
-10 000 m, densities U(1800, 3100)) with its 500 x 500-station survey at
2000 m + N(0, 50 m) (harmonica_gb300.synthetic.layer_topography_1e6, seeded;
synthetic data).  The full survey is 2.5e11 pairs; a STEP is one batch of
the survey (``--stations-per-step`` consecutive stations, default 5000)
against all 1e6 prisms, the batches walking through the survey step after
step.  Per-pair cost is uniform, so pairs/s over batches equals pairs/s over
the full survey.

Keys of the JSON line:

* ``value``: pairs/s of the layer forward with the layer and survey resident
  in HBM, CUDA events around each step's launches on the launching stream,
  L2 flushed between steps.
* ``e2e``: the same through the public drop-in call
  ``layer.prism_layer.gravity(coords, "g_z")`` with host (numpy) buffers:
  host->device copies of the layer and the batch, the kernels and the
  device->host copy of the result inside the timed region.
* ``roofline``: the binding hardware resource of the layer kernel.  The pair
  is evaluated on FP32 float pairs, so the kernel is bound by the FP32 (FMA)
  pipes: ``achieved`` = FP32 lane operations per pair (scalar instructions
  plus twice the packed FADD2/FFMA2/FMUL2) x the kernel's pairs/s, ``peak``
  = 128 FP32 lanes per SM x SMs x the SM clock sampled during the timed
  steps; instruction issue, the other near-binding resource, is reported
  beside it (``issue``: warp instructions per pair x pairs/s against one per
  clock per SM sub-partition).  The instruction, FP64 and DRAM counts per
  pair come from one ncu capture of the same kernel and are used only while
  the kernel sources hash to the value recorded with them (otherwise
  ``stale`` and no fraction).  ``algorithmic`` holds the survey's
  flop convention for the closed form (720 flop per g_z pair: 8 vertices x
  (~16 basic + sqrt + 2 log + 1 atan2) at basic=1, sqrt=4, log=20,
  atan2=30) against the FP64 FMA rate measured live.
* ``all_fields`` / ``potential``: the fused all-field kernel and the
  potential kernel on the same layer (sampled stations).
* ``batched``: the batched workload (256 uneven g_z/g_zz problems) in one
  persistent graph-captured launch per field, against the plain drop-in
  ``prism_gravity`` called once per problem from host buffers.
* ``served``: a Poisson stream of forward solves through the
  continuous-batching server with load shedding, p50/p99 latency over the
  accepted requests, the refused share, and the plain drop-in on the same
  requests one by one from host buffers.
* ``cpu_baseline``: the CPU oracle (a C/OpenMP restatement of the
  reference's per-vertex loop) on all host cores, on a bounded sample of
  stations of the same workload.

``--impl reference`` times the reference's CPU path instead (the oracle port:
the reference's numba + choclo stack is not installable offline) and prints
its own JSON line.
"""

import argparse
import ctypes
import hashlib
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = ("FP64 g_z prism·station pairs/s, served vs plain on 1 GB300 @≤1e-8 rel; "
          "p50/p99 ms")
ARITH = ("FP64 inputs, outputs and accumulation; each pair's closed form evaluated on float "
         "pairs (two FP32 numbers, ~2^-44 relative) with FP64 fallbacks for degenerate "
         "geometry; per-pair error against 50-digit values in tests/test_gpu_truth.py")
WORKLOAD = "layer_topography_1e6: 1000x1000 prisms (200 m grid), 500x500 stations, g_z"
ALGO_FLOP_PER_PAIR_GZ = 720.0
ISSUE_PER_SM_PER_CLOCK = 4  # one warp instruction per clock per SM sub-partition
FP32_LANES_PER_SM_PER_CLOCK = 128  # FMA-heavy + FMA-lite pipes, 16 lanes each per sub-partition

# Kernel sources whose hash keys the ncu counts below.
KERNEL_SOURCES = ("prism_math.cuh", "lean_math.cuh", "lean_packed.cuh", "lean_tables.inc",
                  "forward_core.cuh", "prism_forward.cu")
# ncu counts of the layer g_z kernel (forward_kernel<3, LayerSource, 0>): warp instructions
# (smsp__inst_executed.sum), FP32 lane operations (sm__sass_thread_inst_executed_op_fp32_pred_on
# plus the packed fadd2/ffma2/fmul2 counts once more: two lanes each) and FP64 thread
# instructions (sm__sass_thread_inst_executed_op_fp64_pred_on) per pair, from a capture of a
# 1000-station step (1e9 pairs per launch, two launches); and the DRAM bytes
# (dram__bytes_read.sum + dram__bytes_write.sum) of one launch of the default 5000-station
# step (the layer and the stations are read once; the writes are the chunk partial sums and
# the kernel's few register spills written back from L2).
# Summarised under profiles/; valid for the kernel sources that hash to `sources_sha`.
KERNEL_COUNTS = {
    "sources_sha": "493ff81654005ea1",
    "warp_inst_per_pair": 52.64,
    "fp32_lane_ops_per_pair": 1852.2,
    "fp64_inst_per_pair": 9.40,
    "dram_bytes_default_step": 33995008,  # 25.31 MB read + 8.69 MB written (two launches)
    "default_step_stations": 5000,
    # the same capture's utilisations (fractions of peak over the active cycles)
    "ncu_utilisation": {"issue_active": 0.634, "fma_pipe": 0.695, "fmaheavy_pipe": 0.730,
                        "fmalite_pipe": 0.661, "alu_pipe": 0.345, "fp64_pipe": 0.229},
    "capture": "ncu on GB300: per-pair counts from two launches of a 1000-station step, "
               "DRAM bytes from two launches of the default step (1-pass metrics)",
}


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--stations-per-step", type=int, default=5000)
    p.add_argument("--cpu-sample-stations", type=int, default=32)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-all-fields", action="store_true")
    p.add_argument("--no-batched", action="store_true")
    p.add_argument("--no-served", action="store_true")
    p.add_argument("--all-fields-stations", type=int, default=1000)
    p.add_argument("--workload", default="layer",
                   choices=["layer", "batched", "inversion", "serving", "points", "magnetic",
                            "tesseroids"],
                   help="layer: the 1e6-prism layer with the batched and served blocks "
                        "(default); the others run one secondary workload alone")
    p.add_argument("--batch-problems", type=int, default=256)
    p.add_argument("--no-autotune", action="store_true",
                   help="batched block: run the fixed plan instead of the autotuned shapes")
    p.add_argument("--arrival-seconds", type=float, default=4.0)
    p.add_argument("--rate", type=float, default=200.0)
    p.add_argument("--max-backlog-s", type=float, default=2.0)
    p.add_argument("--plain-sample-seconds", type=float, default=8.0)
    p.add_argument("--serve-round-pairs", type=float, default=None,
                   help="served block: point-prism pairs per round (PrismServer default if unset)")
    p.add_argument("--serve-chunk", type=int, default=None,
                   help="served block: largest prism chunk of a work item (default if unset)")
    return p.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def kernel_sources_sha():
    csrc = os.path.join(HERE, "harmonica_gb300", "csrc")
    h = hashlib.sha256()
    for name in KERNEL_SOURCES:
        with open(os.path.join(csrc, name), "rb") as f:
            h.update(name.encode() + b"\0" + f.read())
    return h.hexdigest()[:16]


class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi during a region."""

    QUERY = (
        "index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
        "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
        "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"
    )

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True,
            )
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        return {
            "sm_mhz": float(np.median(sm)) if sm else None,
            "sm_max_mhz": smax,
            "reasons": sorted(reasons),
            "samples": len(sm),
        }


def bench_lib():
    """The benchmark-support library (include/harmonica_gb300_bench.h)."""
    from harmonica_gb300 import _native

    _native.build()
    _native.lib()  # the bench library resolves the product library's symbols
    lib = ctypes.CDLL(_native.BENCH_LIB_PATH)
    lib.hg_fp64_peak_probe.restype = ctypes.c_int
    lib.hg_fp64_peak_probe.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int,
                                       ctypes.c_void_p]
    return lib


def fp64_peak(torch):
    """Measured FP64 FMA peak (TFLOP/s) of this GPU via hg_fp64_peak_probe."""
    lib = bench_lib()
    n_threads = 152 * 8 * 256
    iters = 4000
    out = torch.empty(n_threads, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    best = 0.0
    for _ in range(4):
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record()
        rc = lib.hg_fp64_peak_probe(out.data_ptr(), n_threads, iters, stream)
        b.record()
        torch.cuda.synchronize()
        assert rc == 0
        flops = n_threads * iters * 16.0
        best = max(best, flops / (a.elapsed_time(b) * 1e-3) / 1e12)
    return best


def cpu_baseline(layer, coords, n_stations, threads):
    """Oracle (per-vertex C/OpenMP restatement of the reference loop) on a sample."""
    from oracle import prism_oracle

    prism_oracle.build_oracle()
    idx = np.linspace(0, coords[0].size - 1, n_stations).astype(np.int64)
    sample = tuple(np.ascontiguousarray(c[idx]) for c in coords)
    t0 = time.perf_counter()
    prism_oracle.layer_gravity(
        sample, layer["easting"], layer["northing"], layer["bottom"], layer["top"],
        layer["density"], "g_z", n_threads=threads,
    )
    dt = time.perf_counter() - t0
    pairs = n_stations * layer["top"].size
    return pairs / dt, dt, pairs


def run_reference(args, rank, world):
    """The reference's CPU path (oracle port) on all host threads."""
    if rank != 0:
        return
    from harmonica_gb300 import synthetic

    layer = synthetic.layer_topography_1e6()
    coords = layer["coordinates"]
    threads = os.cpu_count() or 1
    n = max(1, args.cpu_sample_stations)
    for _ in range(max(0, min(args.warmup, 1))):
        cpu_baseline(layer, coords, max(1, n // 8), threads)
    times = []
    for _ in range(args.steps):
        _, dt, _ = cpu_baseline(layer, coords, n, threads)
        times.append(dt)
    value = float(n * layer["top"].size * len(times) / np.sum(times))
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": value,
        "unit": "pairs/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": float(np.mean(times) * 1e3),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "arith": "FP64 throughout (per-vertex closed form, the reference's algorithm)",
        "data": "synthetic",
        "config": {
            "workload": WORKLOAD,
            "step": f"{n} stations (strided sample of the survey) x 1e6 prisms on the CPU",
        },
        "cpu_baseline": {
            "value": value,
            "unit": "pairs/s",
            "cores": threads,
            "kind": "port",
            "sample": f"{n} of 250000 stations x all 1e6 prisms per step",
        },
        "e2e": {"value": value, "unit": "pairs/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "note": "harmonica's numba+choclo path is not installable offline; the oracle "
                "port (C/OpenMP per-vertex restatement) stands in for it",
    }
    print(json.dumps(line))


# --------------------------------------------------------------------------
# batched block

def batched_block(args, torch, local, timed_replays=2):
    """The batched workload in one persistent graph-captured launch per field
    against (a) the plain drop-in prism_gravity once per problem from host
    buffers, (b) one hg_prism_forward launch per problem on resident inputs."""
    import harmonica_gb300 as hg
    from harmonica_gb300 import synthetic
    from harmonica_gb300.batch import PrismBatch, autotune
    from harmonica_gb300.fields import FIELD_CODES
    from harmonica_gb300.gravity import forward_on_device

    problems = synthetic.batched_problems(args.batch_problems, seed=4)

    def graph_time(batch):
        batch.capture()
        batch.replay()
        torch.cuda.synchronize()
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record()
        for _ in range(timed_replays):
            batch.replay()
        t1.record()
        torch.cuda.synchronize()
        return t0.elapsed_time(t1) * 1e-3 / timed_replays

    tuned = None
    fixed_s = None
    if not args.no_autotune:
        t_tune = time.perf_counter()
        tuned = autotune(problems, repeats=1, cache=None)
        tuned["seconds"] = time.perf_counter() - t_tune
        fixed = PrismBatch(problems, validate=False, shapes=None)
        fixed_s = graph_time(fixed)
        fixed.close()
    batch = PrismBatch(problems, validate=False, shapes=tuned["shapes"] if tuned else None)
    info = batch.info()
    pairs = info["pairs"]
    batched_s = graph_time(batch)
    batched = [o.clone() for o in batch.outputs]

    # (b) one launch per problem on the batch's resident inputs
    keep = batch._keep

    def device_pass():
        outs = []
        for k, p in enumerate(problems):
            e, n, u, soa = keep[4 * k: 4 * k + 4]
            m = np.shape(p["prisms"])[0]
            out, _ = forward_on_device(e, n, u, soa, m, 1 << FIELD_CODES[p["field"]], False)
            outs.append(out)
        return outs

    device_pass()
    torch.cuda.synchronize()
    d0 = time.perf_counter()
    outs = device_pass()
    torch.cuda.synchronize()
    device_s = time.perf_counter() - d0
    worst = 0.0
    for a, b in zip(batched, outs):
        ref = b[0]
        if ref.numel():
            worst = max(worst, (a - ref).abs().max().item() / max(ref.abs().max().item(), 1e-300))
    batch.close()

    # (a) the drop-in from host buffers, problem after problem
    hg.prism_gravity(problems[0]["coordinates"], problems[0]["prisms"], problems[0]["density"],
                     field=problems[0]["field"])
    torch.cuda.synchronize()
    h0 = time.perf_counter()
    for p in problems:
        hg.prism_gravity(p["coordinates"], p["prisms"], p["density"], field=p["field"])
    plain_s = time.perf_counter() - h0
    return {
        "workload": f"{len(problems)} independent problems, prisms log-U[1e3,2e5], stations "
                    "log-U[1e3,5e4], fields g_z/g_zz alternating",
        "pairs_per_pass": pairs,
        "value": pairs / batched_s, "unit": "pairs/s",
        "ms_per_pass": batched_s * 1e3,
        "plain": {"value": pairs / plain_s, "unit": "pairs/s", "ms_per_pass": plain_s * 1e3,
                  "path": "harmonica_gb300.prism_gravity once per problem, numpy inputs"},
        "batched_over_plain": plain_s / batched_s,
        "per_problem_launches": {"value": pairs / device_s, "unit": "pairs/s",
                                 "path": "one hg_prism_forward launch per problem on the "
                                         "resident inputs"},
        "batched_over_per_problem_launches": device_s / batched_s,
        "max_rel_diff_batched_vs_per_problem": worst,
        "work_items": info["items"], "persistent_ctas": info["ctas"],
        "tuned": None if tuned is None else {
            "shapes": tuned["shapes"], "tuning_seconds": tuned["seconds"],
            "candidates_timed": len(tuned["candidates"]),
            "fixed_plan": {"value": pairs / fixed_s, "unit": "pairs/s",
                           "plan": "128 points per CTA, automatic chunk and CTAs"},
            "tuned_over_fixed": fixed_s / batched_s},
        "timed_replays": timed_replays,
    }


# --------------------------------------------------------------------------
# served block

def served_block(args, torch, local):
    """A Poisson stream of forward solves through PrismServer (load shedding
    on), and the plain drop-in on the same requests one by one."""
    import harmonica_gb300 as hg
    from harmonica_gb300 import synthetic
    from harmonica_gb300.serve import PrismServer, ServerOverloaded

    models = synthetic.serving_models()
    stream = synthetic.serving_stream(rate=args.rate, seconds=args.arrival_seconds)
    shape = {}
    if args.serve_round_pairs is not None:
        shape["round_pairs"] = args.serve_round_pairs
    if args.serve_chunk is not None:
        shape["chunk"] = args.serve_chunk
    srv = PrismServer(memory_budget=120e9, max_active=4096, max_backlog_s=args.max_backlog_s,
                      **shape)
    for k in range(8):
        srv.register_layer(f"layer{k}", models[k][0], models[k][1])
    coords_of = [synthetic.serving_request_coordinates(r, models[r["model"]][2]) for r in stream]
    # warm the kernels of the three fields outside the measured stream, with
    # requests large enough (~1e9 pairs) for each field's rate to be timed
    srv.max_backlog_s = None
    big = max(range(8), key=lambda k: models[k][0].shape[0])
    side = models[big][2]
    n_warm = int(min(20000, max(1000, 1e9 / models[big][0].shape[0])))
    rw = np.random.default_rng(99)
    warm_coords = (rw.uniform(0, side, n_warm), rw.uniform(0, side, n_warm),
                   rw.uniform(100, 3000, n_warm))
    for f in ("g_z", "potential", "g_zz"):
        srv.submit(warm_coords, f, layer=f"layer{big}").result()
    srv.max_backlog_s = args.max_backlog_s
    offered = sum(r["n_stations"] * models[r["model"]][0].shape[0] for r in stream)
    futures = []
    t0 = time.perf_counter()
    for r, coords in zip(stream, coords_of):
        delay = r["t"] - (time.perf_counter() - t0)
        if delay > 0:
            time.sleep(delay)
        if r["resident"]:
            f = srv.submit(coords, r["field"], layer=f"layer{r['model']}")
        else:
            f = srv.submit(coords, r["field"], prisms=models[r["model"]][0],
                           density=models[r["model"]][1])
        futures.append((f, r, time.perf_counter()))
    accepted = [(f, r, ts) for f, r, ts in futures
                if not (f.done() and isinstance(f.exception(), ServerOverloaded))]
    done_pairs = 0.0
    for f, r, ts in accepted:
        f.result()  # accepted requests all finish (the backlog is bounded)
        done_pairs += r["n_stations"] * models[r["model"]][0].shape[0]
    st = srv.stats()
    mine = {id(f) for f, _, _ in accepted}
    finished = [req for req in srv.completed if id(req.future) in mine]
    latencies = np.array([req.t_done - req.t_submit for req in finished])
    elapsed = max(req.t_done for req in finished) - t0
    srv.close(drain=True, timeout=60)
    fields = {}
    for f, r, ts in accepted:
        fields[r["field"]] = fields.get(r["field"], 0) + 1

    # the plain drop-in on the same requests the server accepted, one by one in
    # arrival order (a bounded sample): the same mix of sizes and fields
    plain_pairs, plain_s, n_plain = 0.0, 0.0, 0
    coords_by_id = {id(r): c for r, c in zip(stream, coords_of)}
    for _, r, _ in accepted:
        coords = coords_by_id[id(r)]
        prisms, density, _ = models[r["model"]]
        torch.cuda.synchronize()
        a = time.perf_counter()
        hg.prism_gravity(coords, prisms, density, field=r["field"])
        plain_s += time.perf_counter() - a
        plain_pairs += r["n_stations"] * prisms.shape[0]
        n_plain += 1
        if plain_s >= args.plain_sample_seconds:
            break
    served_rate = done_pairs / elapsed
    plain_rate = plain_pairs / plain_s
    return {
        "workload": f"Poisson {args.rate}/s for {args.arrival_seconds} s, prisms log-U[1e3,1e6], "
                    "stations log-U[1e3,2.5e5], fields g_z/potential/g_zz, 30% on 8 resident "
                    "layers, 120 GB budget",
        "requests": len(stream),
        "offered_pairs_per_s": offered / args.arrival_seconds,
        "accepted": len(accepted), "refused": st["rejected"],
        "refused_share": st["rejected"] / max(len(stream), 1),
        "max_backlog_s": args.max_backlog_s,
        "completed": len(latencies),
        "value": served_rate, "unit": "pairs/s",
        "p50_ms": float(np.percentile(latencies, 50) * 1e3) if latencies.size else None,
        "p99_ms": float(np.percentile(latencies, 99) * 1e3) if latencies.size else None,
        "latency_over": "every accepted request (all finished); refused requests are answered "
                        "at once with ServerOverloaded",
        "measured_seconds": elapsed, "rounds": st["rounds"],
        "round_pairs": srv.round_pairs, "chunk": srv.max_chunk,
        "accepted_fields": fields,
        "plain": {"value": plain_rate, "unit": "pairs/s", "requests": n_plain,
                  "path": "harmonica_gb300.prism_gravity once per request, numpy inputs, the "
                          "accepted requests in arrival order"},
        "served_over_plain": served_rate / plain_rate,
    }


# --------------------------------------------------------------------------
# secondary workloads (run alone with --workload)

def run_batched(args, rank, world, local):
    import torch

    from harmonica_gb300 import _native

    _native.build()
    torch.cuda.set_device(local)
    blk = batched_block(args, torch, local, timed_replays=max(1, args.steps))
    if rank == 0:
        print(json.dumps({"metric": "FP64 g_z/g_zz prism-station pairs/s, batched persistent "
                                    "launch", "value": blk["value"], "unit": "pairs/s",
                          "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
                          "higher_is_better": True, "dtype": "f64", "arith": ARITH,
                          "data": "synthetic", "batched": blk,
                          "gpu_launches": 3 * args.steps}))


def run_serving(args, rank, world, local):
    import torch

    from harmonica_gb300 import _native

    _native.build()
    torch.cuda.set_device(local)
    blk = served_block(args, torch, local)
    if rank == 0:
        print(json.dumps({"metric": "served FP64 pairs/s and latency, Poisson stream of "
                                    "forward solves", "value": blk["value"], "unit": "pairs/s",
                          "n_gpus": world, "steps": 1, "warmup": 0, "higher_is_better": True,
                          "dtype": "f64", "arith": ARITH, "data": "synthetic", "served": blk}))


def run_inversion(args, rank, world, local):
    """Basement-inversion step: FP64 forward + adjoint (density, bottom) of a 200x200 layer."""
    import torch

    import harmonica_gb300 as hg
    from harmonica_gb300 import _native, synthetic

    _native.build()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    L = synthetic.basement_layer()
    T = lambda a: torch.tensor(a, dtype=torch.float64, device=dev)  # noqa: E731
    coords = tuple(T(c) for c in L["coordinates"])
    ce, cn = T(L["easting"]), T(L["northing"])
    with torch.no_grad():
        true_gz = hg.layer_gravity_torch(coords, ce, cn, T(L["bottom"]), T(L["top"]),
                                         T(L["density"]))
    rng = np.random.default_rng(L["noise_seed"])
    data = true_gz + T(rng.normal(0.0, 0.1, true_gz.numel()))
    start = T(np.full_like(L["bottom"], -3000.0))

    def step():
        bottom = start.clone().requires_grad_(True)
        rho = T(L["density"]).requires_grad_(True)
        gz = hg.layer_gravity_torch(coords, ce, cn, bottom, T(L["top"]), rho)
        loss = 0.5 * ((gz - data) ** 2).sum()
        loss.backward()
        return loss.detach(), bottom.grad, rho.grad

    for _ in range(max(1, args.warmup)):
        step()
    torch.cuda.synchronize()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record()
    for _ in range(args.steps):
        loss, gb, gr = step()
    t1.record()
    torch.cuda.synchronize()
    step_s = t0.elapsed_time(t1) * 1e-3 / args.steps
    pairs = coords[0].numel() * L["bottom"].size
    if rank != 0:
        return
    print(json.dumps({
        "metric": "basement inversion step (FP64 g_z forward + adjoint d/drho, d/dbottom)",
        "value": pairs / step_s, "unit": "forward pairs/s", "ms_per_step": step_s * 1e3,
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
        "dtype": "f64", "arith": ARITH, "data": "synthetic",
        "config": {"workload": "200x200 layer (500 m), tops 0, smooth bottoms N(-3000,800), "
                               "contrast -400, 100x100 stations at 500 m",
                   "pairs_per_forward": pairs, "loss": float(loss),
                   "grad_bottom_norm": float(gb.norm()), "grad_density_norm": float(gr.norm())},
        "gpu_launches": 4 * args.steps,
    }))


def run_points(args, rank, world, local):
    """Point masses (Cartesian g_z): 1e6 masses under the 500 x 500 survey."""
    import torch

    from harmonica_gb300 import _native, synthetic
    from harmonica_gb300.gravity import _ptr

    _native.build()
    lib = _native.lib()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    L = synthetic.layer_topography_1e6()
    prisms, density = synthetic.layer_to_prisms(L)
    # one point mass per prism, at its centre, with its mass
    pe = 0.5 * (prisms[:, 0] + prisms[:, 1])
    pn = 0.5 * (prisms[:, 2] + prisms[:, 3])
    pu = 0.5 * (prisms[:, 4] + prisms[:, 5])
    vol = (prisms[:, 1] - prisms[:, 0]) * (prisms[:, 3] - prisms[:, 2]) * (prisms[:, 5] - prisms[:, 4])
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).to(dev)  # noqa: E731
    p = [T(pe), T(pn), T(pu), T(vol * density)]
    c = [T(x) for x in L["coordinates"]]
    B = 20000
    out = torch.empty(B, dtype=torch.float64, device=dev)
    ws = _native.ctypes.c_size_t(0)
    _native.check(lib.hg_point_forward_workspace(B, pe.size, _native.ctypes.byref(ws)))
    work = torch.empty(max(1, (ws.value + 7) // 8), dtype=torch.float64, device=dev)

    def step(s):
        lo = (s * B) % (c[0].numel() - B)
        _native.check(lib.hg_point_forward(
            _ptr(c[0][lo:]), _ptr(c[1][lo:]), _ptr(c[2][lo:]), B, _ptr(p[0]), _ptr(p[1]),
            _ptr(p[2]), _ptr(p[3]), pe.size, 0, 3, _ptr(out), _ptr(work), ws.value,
            torch.cuda.current_stream().cuda_stream))

    for s in range(args.warmup):
        step(s)
    torch.cuda.synchronize()
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    a.record()
    for s in range(args.steps):
        step(args.warmup + s)
    b.record()
    torch.cuda.synchronize()
    sec = a.elapsed_time(b) * 1e-3 / args.steps
    if rank == 0:
        print(json.dumps({"metric": "FP64 g_z point-mass pairs/s (Cartesian)",
                          "value": B * pe.size / sec, "unit": "pairs/s", "ms_per_step": sec * 1e3,
                          "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
                          "dtype": "f64", "data": "synthetic",
                          "config": {"workload": "1e6 point masses (prism centres of the 1e6 "
                                                 "layer), 20000 stations per step"},
                          "gpu_launches": 2 * args.steps}))


def run_magnetic(args, rank, world, local):
    """Prism magnetics (b_e, b_n, b_u together) on the 1e6-prism layer."""
    import torch

    from harmonica_gb300 import _native, synthetic
    from harmonica_gb300.gravity import _ptr

    _native.build()
    lib = _native.lib()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    L = synthetic.layer_topography_1e6()
    prisms, _ = synthetic.layer_to_prisms(L)
    rng = np.random.default_rng(8)
    mag = [rng.uniform(-1, 1, prisms.shape[0]) for _ in range(3)]
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).to(dev)  # noqa: E731
    m = prisms.shape[0]
    soa = torch.empty((9, m), dtype=torch.float64, device=dev)
    aos, me, mn, mu = T(prisms), T(mag[0]), T(mag[1]), T(mag[2])
    stream = torch.cuda.current_stream().cuda_stream
    _native.check(lib.hg_pack_prisms_magnetic(_ptr(aos), _ptr(me), _ptr(mn), _ptr(mu), m,
                                              _ptr(soa), m, stream))
    c = [T(x) for x in L["coordinates"]]
    B = 1000
    out = torch.empty((3, B), dtype=torch.float64, device=dev)
    ws = _native.ctypes.c_size_t(0)
    _native.check(lib.hg_prism_magnetic_workspace(B, m, 3, _native.ctypes.byref(ws)))
    work = torch.empty(max(1, (ws.value + 7) // 8), dtype=torch.float64, device=dev)

    def step(s):
        lo = (s * B) % (c[0].numel() - B)
        _native.check(lib.hg_prism_magnetic(_ptr(c[0][lo:]), _ptr(c[1][lo:]), _ptr(c[2][lo:]),
                                            B, _ptr(soa), m, m, 3, _ptr(out), _ptr(work),
                                            ws.value, torch.cuda.current_stream().cuda_stream))

    for s in range(args.warmup):
        step(s)
    torch.cuda.synchronize()
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    a.record()
    for s in range(args.steps):
        step(args.warmup + s)
    b.record()
    torch.cuda.synchronize()
    sec = a.elapsed_time(b) * 1e-3 / args.steps
    if rank == 0:
        print(json.dumps({"metric": "FP64 prism magnetic pairs/s (b_e, b_n, b_u per pair)",
                          "value": B * m / sec, "unit": "pairs/s", "ms_per_step": sec * 1e3,
                          "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
                          "dtype": "f64", "arith": ARITH, "data": "synthetic",
                          "config": {"workload": "1e6-prism layer, magnetization U(-1,1) A/m, "
                                                 "1000 stations per step"},
                          "gpu_launches": 2 * args.steps}))


# Per-pair instruction counts of the tesseroid forward kernel on the Andes layer, from
# ncu on one bench launch (smsp__inst_executed.sum and
# sm__sass_thread_inst_executed_op_fp64_pred_on.sum over its 3825 x 93121 pairs), and the
# DRAM bytes of that launch; summarised under profiles/.
WARP_INST_PER_TESS_PAIR = 20.4
FP64_INST_PER_TESS_PAIR = 2.56
TRAFFIC_BYTES_TESS_STEP = 46889728 + 35952384


def run_tesseroids(args, rank, world, local):
    """Tesseroid layer g_z: the gallery's Andes tesseroid layer (93,121 tesseroids,
    3,825 points 10 km above the reference), one full forward per step."""
    import torch

    import harmonica_gb300 as hg
    from harmonica_gb300 import _native, synthetic, tesseroid

    _native.build()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    L = synthetic.tesseroid_layer_andes()
    tess, dens, coords = L["tesseroids"], L["density"], L["coordinates"]
    if world > 1:  # each rank takes a contiguous share of the points (no collective)
        lo, hi = rank * coords[0].size // world, (rank + 1) * coords[0].size // world
        coords = tuple(c[lo:hi] for c in coords)
    n_obs, m = coords[0].size, tess.shape[0]
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).to(dev)  # noqa: E731
    c = [T(x) for x in coords]
    t_dev, rho = T(tess), T(dens)
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 8, dtype=torch.float64, device=dev)

    def step():
        return tesseroid.tesseroid_gravity_device(c[0], c[1], c[2], t_dev, rho, "g_z",
                                                  status=status)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    peak = fp64_peak(torch)
    sampler = ClockSampler(local)
    sampler.start()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    t_wall = time.perf_counter()
    for s in range(args.steps):
        flush.fill_(float(s))  # L2 flush between timed steps (outside the events)
        starts[s].record()
        out = step()
        ends[s].record()
    torch.cuda.synchronize()
    wall = time.perf_counter() - t_wall
    clocks = sampler.stop()
    if int(status.item()) != 0:
        raise RuntimeError("tesseroid forward reported an overflow on the bench workload")
    step_ms = [a.elapsed_time(b) for a, b in zip(starts, ends)]
    dev_time = sum(step_ms) * 1e-3
    pairs = n_obs * m * args.steps
    if world > 1:
        t = torch.tensor([dev_time, float(pairs)], dtype=torch.float64, device=dev)
        if not torch.distributed.is_initialized():
            torch.distributed.init_process_group("nccl", device_id=dev)
        torch.distributed.all_reduce(t[:1], op=torch.distributed.ReduceOp.MAX)
        torch.distributed.all_reduce(t[1:])
        dev_time, pairs = float(t[0].item()), int(t[1].item())
    value = pairs / dev_time

    e2e = None
    if not args.no_e2e:
        hg.tesseroid_gravity(coords, tess, dens, field="g_z")  # warm
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            res = hg.tesseroid_gravity(coords, tess, dens, field="g_z")
        e2e_time = time.perf_counter() - t0
        e2e = {"value": pairs / e2e_time, "unit": "pairs/s",
               "h2d_bytes_per_step": 8 * (3 * n_obs + 6 * m + m), "d2h_bytes_per_step": 8 * n_obs,
               "path": "harmonica_gb300.tesseroid_gravity with numpy inputs (checks, "
                       "points-inside test on the GPU, copies, forward)"}
        ref_dev = out.cpu().numpy()
        if not np.allclose(res, ref_dev, rtol=1e-12, atol=0):
            raise RuntimeError("device and end-to-end tesseroid results differ")

    base = None
    if rank == 0 and not args.no_cpu_baseline:
        from oracle import tesseroid_oracle

        idx = np.linspace(0, n_obs - 1, max(args.cpu_sample_stations, 512)).astype(int)
        sub = tuple(x[idx] for x in coords)
        t0 = time.perf_counter()
        tesseroid_oracle.tesseroid_gravity(sub, tess, dens, "g_z")
        dt = time.perf_counter() - t0
        base = {"value": idx.size * m / dt, "unit": "pairs/s", "cores": os.cpu_count() or 1,
                "kind": "port",
                "sample": f"{idx.size} strided points x all {m} tesseroids ({dt:.1f} s, "
                          "OpenMP over points)"}
    if rank != 0:
        return
    kernel_rate = n_obs * m / (dev_time / args.steps)
    n_sms = torch.cuda.get_device_properties(dev).multi_processor_count
    sm_hz = (clocks.get("sm_mhz") or clocks.get("sm_max_mhz") or 0.0) * 1e6
    issue_peak = ISSUE_PER_SM_PER_CLOCK * n_sms * sm_hz
    issue_rate = WARP_INST_PER_TESS_PAIR * kernel_rate
    roof = {"bound": "instruction issue", "achieved": issue_rate / 1e9,
            "peak": issue_peak / 1e9 if issue_peak else None, "unit": "G warp-instructions/s",
            "frac": issue_rate / issue_peak if issue_peak else None,
            "warp_inst_per_pair": WARP_INST_PER_TESS_PAIR,
            "peak_source": "4 warp instructions per clock per SM x SMs x sampled SM clock",
            "traffic": TRAFFIC_BYTES_TESS_STEP,
            "fp64": {"inst_per_pair": FP64_INST_PER_TESS_PAIR,
                     "pipe_frac": FP64_INST_PER_TESS_PAIR * kernel_rate / (peak * 1e12 / 2.0),
                     "peak": peak, "unit": "TFLOP/s",
                     "peak_source": "measured live: hg_fp64_peak_probe (FP64 FMA chains)"}}
    print(json.dumps({
        "metric": "FP64 tesseroid g_z pairs/s (points x tesseroids, adaptive GLQ)",
        "value": value, "unit": "pairs/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": wall / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": f"tesseroid layer, Andes region at 0.1 deg ({m} tesseroids), "
                               f"{n_obs} points 10 km above the WGS84 reference",
                   "l2": "flushed between timed steps (256 MB write)"},
        "roofline": roof, "cpu_baseline": base, "e2e": e2e,
        "gpu_launches": 4 * args.steps, "clocks": clocks, "step_ms": step_ms,
    }))


# --------------------------------------------------------------------------
# the headline

def layer_roofline(torch, dev, kernel_pairs_per_s, clocks, stations_per_step, algo_bytes):
    """Roofline of the layer g_z kernel on its binding resource (the FP32
    pipes), with instruction issue and the algorithmic FP64 figure beside it."""
    peak = fp64_peak(torch)
    sha = kernel_sources_sha()
    counts = KERNEL_COUNTS
    fresh = counts["sources_sha"] == sha and counts["warp_inst_per_pair"] is not None
    n_sms = torch.cuda.get_device_properties(dev).multi_processor_count
    sm_hz = (clocks.get("sm_mhz") or clocks.get("sm_max_mhz") or 0.0) * 1e6
    issue_peak = ISSUE_PER_SM_PER_CLOCK * n_sms * sm_hz
    algo = ALGO_FLOP_PER_PAIR_GZ * kernel_pairs_per_s / 1e12
    fp32_peak = FP32_LANES_PER_SM_PER_CLOCK * n_sms * sm_hz
    roof = {
        "bound": "fp32 pipe",
        "unit": "T FP32 lane-ops/s",
        "peak": fp32_peak / 1e12 if fp32_peak else None,
        "peak_source": "128 FP32 lanes per clock per SM x SMs x the SM clock sampled during "
                       "the timed steps (no FP32 figure in the measured peaks)",
        "kernel_sources_sha": sha,
        "counts_from": counts["capture"] if fresh else None,
        "stale": not fresh,
        "achieved": None, "frac": None, "traffic": None,
        "algorithmic": {
            "flop_per_pair": ALGO_FLOP_PER_PAIR_GZ,
            "achieved": algo, "unit": "TFLOP/s",
            "fp64_peak": peak, "fp64_peak_source": "measured live: hg_fp64_peak_probe "
                                                   "(FP64 FMA chains)",
            "ratio_to_fp64_peak": algo / peak,
            "note": "the convention's flops per pair over the FP64 peak: the kernel evaluates "
                    "the pair on float pairs and runs far fewer FP64 instructions, so this "
                    "ratio rates the algorithm, not the hardware",
        },
    }
    if fresh:
        issue_rate = counts["warp_inst_per_pair"] * kernel_pairs_per_s
        fp32_rate = counts["fp32_lane_ops_per_pair"] * kernel_pairs_per_s
        same_step = stations_per_step == counts["default_step_stations"]
        roof.update(achieved=fp32_rate / 1e12,
                    frac=fp32_rate / fp32_peak if fp32_peak else None,
                    fp32_lane_ops_per_pair=counts["fp32_lane_ops_per_pair"],
                    issue={"achieved": issue_rate / 1e9, "unit": "G warp-instructions/s",
                           "peak": issue_peak / 1e9 if issue_peak else None,
                           "frac": issue_rate / issue_peak if issue_peak else None,
                           "peak_source": "4 warp instructions per clock per SM x SMs x the "
                                          "SM clock sampled during the timed steps"},
                    warp_inst_per_pair=counts["warp_inst_per_pair"],
                    ncu_utilisation=counts["ncu_utilisation"],
                    traffic=counts["dram_bytes_default_step"] if same_step else None,
                    algorithmic_bytes=algo_bytes,
                    fp64={"inst_per_pair": counts["fp64_inst_per_pair"],
                          "pipe_frac": counts["fp64_inst_per_pair"] * kernel_pairs_per_s
                          / (peak * 1e12 / 2.0)})
    return roof


def main():
    args = parse_args()
    rank, world, local = dist_env()
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    secondary = {"batched": run_batched, "inversion": run_inversion, "serving": run_serving,
                 "points": run_points, "magnetic": run_magnetic, "tesseroids": run_tesseroids}
    if args.workload in secondary:
        secondary[args.workload](args, rank, world, local)
        return

    import torch

    import harmonica_gb300 as hg
    from harmonica_gb300 import _native, synthetic
    from harmonica_gb300.layer import layer_forward_device

    _native.build()
    lib = _native.lib()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=dev)

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    layer = synthetic.layer_topography_1e6()
    coords = layer["coordinates"]
    n_total = coords[0].size
    B = args.stations_per_step
    mask = 1 << 3  # g_z
    n_prisms = layer["top"].size

    # resident layer and survey
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).to(dev)  # noqa: E731
    ce, cn = T(layer["easting"]), T(layer["northing"])
    bt, tp, rho = T(layer["bottom"]), T(layer["top"]), T(layer["density"])
    de, dn, du = (T(c) for c in coords)

    # each rank walks its own batches of the survey (no collective on the data path)
    def batch(step):
        k = (step * world + rank) % ((n_total + B - 1) // B)
        lo = k * B
        hi = min(lo + B, n_total)
        return lo, hi

    ws_bytes = _native.ctypes.c_size_t(0)
    _native.check(lib.hg_layer_forward_workspace(B, ce.numel(), cn.numel(), mask,
                                                 _native.ctypes.byref(ws_bytes)))
    launches_per_step = 2 if ws_bytes.value else 1

    flush = torch.empty(256 * 1024 * 1024 // 8, dtype=torch.float64, device=dev)

    def step_device(step, field_mask=mask):
        lo, hi = batch(step)
        return layer_forward_device(de[lo:hi], dn[lo:hi], du[lo:hi], ce, cn, bt, tp, rho,
                                    field_mask, 0.0)

    for s in range(args.warmup):
        step_device(s)
    torch.cuda.synchronize()

    sampler = ClockSampler(local)
    sampler.start()
    barrier()
    torch.cuda.synchronize()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    pairs = 0
    t_wall = time.perf_counter()
    for s in range(args.steps):
        flush.fill_(float(s))  # L2 flush between timed steps (outside the events)
        starts[s].record()
        out = step_device(args.warmup + s)
        ends[s].record()
        lo, hi = batch(args.warmup + s)
        pairs += (hi - lo) * n_prisms
    torch.cuda.synchronize()
    barrier()
    wall = time.perf_counter() - t_wall
    clocks = sampler.stop()
    step_ms = [a.elapsed_time(b) for a, b in zip(starts, ends)]
    dev_time = sum(step_ms) * 1e-3
    if world > 1:
        t = torch.tensor([dev_time], dtype=torch.float64, device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        dev_time = float(t.item())
        pt = torch.tensor([float(pairs)], dtype=torch.float64, device=dev)
        torch.distributed.all_reduce(pt)
        pairs = int(pt.item())
    value = pairs / dev_time
    del out

    # end-to-end through the public drop-in API with host buffers
    e2e = None
    if not args.no_e2e:
        L = hg.prism_layer((layer["easting"], layer["northing"]), layer["top"], layer["bottom"],
                           properties={"density": layer["density"]})
        host_batches = []
        for s in range(args.steps):
            lo, hi = batch(args.warmup + s)
            host_batches.append(tuple(np.ascontiguousarray(c[lo:hi]) for c in coords))
        L.prism_layer.gravity(host_batches[0], field="g_z")  # warm
        barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e2e_pairs = 0
        for hb in host_batches:
            L.prism_layer.gravity(hb, field="g_z")
            e2e_pairs += hb[0].size * n_prisms
        torch.cuda.synchronize()
        e2e_time = time.perf_counter() - t0
        if world > 1:
            t = torch.tensor([e2e_time], dtype=torch.float64, device=dev)
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            e2e_time = float(t.item())
            e2e_pairs *= world
        h2d = 8 * (3 * B + layer["easting"].size + layer["northing"].size + 3 * n_prisms)
        e2e = {"value": e2e_pairs / e2e_time, "unit": "pairs/s", "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": 8 * B,
               "path": "prism_layer(...).prism_layer.gravity(coords, 'g_z'), numpy inputs"}

    def sampled_rate(field_mask, label):
        """One forward call of `field_mask` on sampled stations of the layer (two
        launches for the potential or the ten fields: edge-log terms, then face terms)."""
        nb = min(args.all_fields_stations, n_total)
        lo = rank * nb % n_total
        sl = slice(lo, lo + nb)
        layer_forward_device(de[sl], dn[sl], du[sl], ce, cn, bt, tp, rho, field_mask, 0.0)
        torch.cuda.synchronize()
        a0 = torch.cuda.Event(enable_timing=True)
        a1 = torch.cuda.Event(enable_timing=True)
        a0.record()
        layer_forward_device(de[sl], dn[sl], du[sl], ce, cn, bt, tp, rho, field_mask, 0.0)
        a1.record()
        torch.cuda.synchronize()
        sec = a0.elapsed_time(a1) * 1e-3
        return {"value": nb * n_prisms / sec, "unit": f"pairs/s ({label})",
                "sample": f"{nb} stations x all 1e6 prisms, one call (edge-log and face "
                          "launches)", "ms": sec * 1e3}

    all_fields = potential = None
    if not args.no_all_fields:
        all_fields = sampled_rate(0x3FF, "all 10 fields per pair")
        all_fields["field_values_per_s"] = 10 * all_fields["value"]
        potential = sampled_rate(1 << 0, "potential")

    base = None
    if rank == 0 and not args.no_cpu_baseline:
        rate, dt, sample_pairs = cpu_baseline(layer, coords, args.cpu_sample_stations,
                                              os.cpu_count() or 1)
        base = {"value": rate, "unit": "pairs/s", "cores": os.cpu_count() or 1, "kind": "port",
                "sample": f"{args.cpu_sample_stations} strided stations x all 1e6 prisms "
                          f"({sample_pairs:.3g} pairs, {dt:.1f} s)"}

    batched = served = None
    if rank == 0 and not args.no_batched:
        batched = batched_block(args, torch, local)
    if rank == 0 and not args.no_served:
        served = served_block(args, torch, local)

    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return
    avg_launch_s = dev_time / args.steps
    kernel_pairs_per_s = (pairs / world / args.steps) / avg_launch_s
    line = {
        "metric": METRIC,
        "value": value,
        "unit": "pairs/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": wall / args.steps * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "arith": ARITH,
        "data": "synthetic",
        "config": {
            "workload": WORKLOAD,
            "step": f"{B} consecutive survey stations x all 1e6 prisms ({B * n_prisms:.3g} pairs)",
            "full_survey_steps": (n_total + B - 1) // B,
            "l2": "flushed between timed steps (256 MB write)",
            "parallelism": f"stations sharded over {world} GPU(s), no collective",
        },
        # algorithmic bytes of a step: the layer (centres, top, bottom, density)
        # and the step's stations read once, its results written once
        "roofline": layer_roofline(torch, dev, kernel_pairs_per_s, clocks, B,
                                   8 * (layer["easting"].size + layer["northing"].size
                                        + 3 * n_prisms + 3 * B + B)),
        "cpu_baseline": base,
        "e2e": e2e,
        "served": served,
        "batched": batched,
        "all_fields": all_fields,
        "potential": potential,
        "gpu_launches": launches_per_step * args.steps,
        "clocks": clocks,
        "step_ms": step_ms,
    }
    print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
