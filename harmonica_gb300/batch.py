"""
Many independent prism forward problems in one persistent launch.

:class:`PrismBatch` wraps the C ABI ``hg_batch_*``: it keeps every problem's
inputs and outputs resident on the device, builds the work list once, and
runs it with one memset, one launch per field present (two for the
potential) and one reduction on the current stream — directly or replayed from a captured CUDA graph.
:func:`autotune` picks, per field, the shape of the work (observation points
per CTA and per work item, which is also the prism tile staged in shared
memory; prisms per work item; persistent CTAs) by timing candidate shapes on
a sample of the real problems, and caches the choice (keyed by device and a
coarse signature of the batch) in a JSON file.

This replaces a loop of ``harmonica.prism_gravity`` calls, one per problem
(``src/harmonica/_forward/prisms/gravity.py:51-236``).
"""

import ctypes
import hashlib
import json
import os
import warnings

import numpy as np

from . import _native
from .fields import FIELD_CODES, TENSOR_FIELDS
from .gravity import _prepare, pack_prisms

DEFAULT_CACHE = os.path.join(os.path.expanduser("~"), ".cache", "harmonica_gb300",
                             "batch_tuning.json")


class PrismBatch:
    """
    A batch of ``(coordinates, prisms, density, field)`` problems resident on
    one GPU.

    Parameters
    ----------
    problems : list of dict
        Each with ``coordinates`` (3 arrays), ``prisms`` ((M, 6) array),
        ``density`` ((M,) array) and ``field`` (one of the ten field names).
        Host arrays are copied to the device once; torch CUDA tensors of
        float64 are used in place.
    chunk_prisms, n_ctas : int
        Work-list shape for every field (0 = automatic, 128 points per CTA).
    shapes : "auto", dict or None
        Per-field shapes ``{field: {"chunk_prisms", "points_per_cta",
        "n_ctas"}}`` (as :func:`autotune` returns them); fields not listed
        take ``chunk_prisms`` / ``n_ctas``.  ``"auto"`` (the default) runs
        :func:`autotune` on the problems (cached per device and batch
        signature) unless ``chunk_prisms`` or ``n_ctas`` is given; ``None``
        takes the fixed plan (128 points per CTA, ``chunk_prisms`` and
        ``n_ctas``).
    check_singular : bool
        Scan tensor-field problems for points on singular edges/vertices
        (one flag per problem, see :meth:`singular`).
    """

    def __init__(self, problems, chunk_prisms=0, n_ctas=0, check_singular=False, device=None,
                 validate=True, shapes="auto"):
        import torch

        from .gravity import _device

        self.torch = torch
        self.device = _device(device)
        if isinstance(shapes, str):
            if shapes != "auto":
                raise ValueError(f"shapes must be 'auto', a dict or None, not {shapes!r}")
            explicit = chunk_prisms or n_ctas
            shapes = None if explicit or not problems else autotune(
                problems, device=self.device)["shapes"]
        self.shapes = shapes
        self.lib = _native.lib()
        self.fields = []
        self.shapes = []
        self._keep = []
        probs = (_native.HgProblem * max(len(problems), 1))()
        with torch.cuda.device(self.device):
            self.flags = torch.zeros(max(len(problems), 1), dtype=torch.int32,
                                     device=self.device)
            self.outputs = []
            for k, pb in enumerate(problems):
                field = pb["field"]
                if field not in FIELD_CODES:
                    raise ValueError(f"Gravitational field {field} not recognized")
                e, n, u, soa, m, shape = self._stage(pb, validate)
                out = torch.empty(e.numel(), dtype=torch.float64, device=self.device)
                self._keep += [e, n, u, soa]
                self.outputs.append(out)
                self.fields.append(field)
                self.shapes.append(shape)
                p = probs[k]
                p.obs_e, p.obs_n, p.obs_u = e.data_ptr(), n.data_ptr(), u.data_ptr()
                p.n_obs = e.numel()
                p.prisms_soa = soa.data_ptr()
                p.prism_stride = soa.shape[1]
                p.n_prisms = m
                p.field = FIELD_CODES[field]
                p.check_singular = int(check_singular and field in TENSOR_FIELDS)
                p.out = out.data_ptr() if out.numel() else None
                p.singular_flag = self.flags[k:].data_ptr()
            handle = ctypes.c_void_p()
            table = (_native.HgBatchShape * len(FIELD_CODES))()
            for name, code in FIELD_CODES.items():
                shape = (shapes or {}).get(name, {})
                table[code].chunk_prisms = int(shape.get("chunk_prisms", chunk_prisms))
                table[code].points_per_cta = int(shape.get("points_per_cta", 128))
                table[code].n_ctas = int(shape.get("n_ctas", n_ctas))
            _native.check(self.lib.hg_batch_create_shaped(probs, len(problems), table,
                                                          ctypes.byref(handle)))
            self.handle = handle
            ws = ctypes.c_size_t(0)
            _native.check(self.lib.hg_batch_workspace(self.handle, ctypes.byref(ws)))
            self.workspace_bytes = ws.value
            self.workspace = torch.empty((ws.value + 7) // 8, dtype=torch.float64,
                                         device=self.device)
        self.graph = None

    def _stage(self, pb, validate):
        torch = self.torch
        dev = self.device
        coords = pb["coordinates"]
        if isinstance(coords[0], torch.Tensor):
            e, n, u = (c.to(dev, torch.float64).contiguous().ravel() for c in coords[:3])
            if not e.numel() == n.numel() == u.numel():
                raise ValueError("The coordinates of a problem must have the same number of "
                                 "elements.")
            shape = tuple(coords[0].shape)
        else:
            cast, host_coords, _, _ = _prepare(coords, np.zeros((0, 6)), np.zeros(0), True)
            e, n, u = (torch.from_numpy(c).to(dev) for c in host_coords)
            shape = cast.shape
        prisms, density = pb["prisms"], pb["density"]
        if isinstance(prisms, torch.Tensor):
            pr = prisms.to(dev, torch.float64).contiguous()
            rho = density.to(dev, torch.float64).contiguous()
        else:
            _, _, p_np, d_np = _prepare(([0.0], [0.0], [0.0]), prisms, density, not validate)
            pr = torch.from_numpy(np.ascontiguousarray(p_np)).to(dev)
            rho = torch.from_numpy(np.ascontiguousarray(d_np)).to(dev)
        soa = pack_prisms(pr, rho)
        return e, n, u, soa, pr.shape[0], shape

    # ------------------------------------------------------------------
    def info(self):
        n_items, n_ctas, pairs = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_double()
        _native.check(self.lib.hg_batch_info(self.handle, ctypes.byref(n_items),
                                             ctypes.byref(n_ctas), ctypes.byref(pairs)))
        return {"items": n_items.value, "ctas": n_ctas.value, "pairs": pairs.value}

    def run(self):
        """Queue the batch on the current stream (asynchronous)."""
        stream = self.torch.cuda.current_stream(self.device).cuda_stream
        _native.check(self.lib.hg_batch_run(self.handle, self.workspace.data_ptr(),
                                            self.workspace_bytes, stream))

    def capture(self):
        """Capture one run in a CUDA graph; :meth:`replay` then re-runs it."""
        torch = self.torch
        with torch.cuda.device(self.device):
            s = torch.cuda.Stream()
            s.wait_stream(torch.cuda.current_stream())
            with torch.cuda.stream(s):
                self.run()  # warm-up outside the capture
            torch.cuda.current_stream().wait_stream(s)
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g):
                self.run()
            self.graph = g
        return g

    def replay(self):
        if self.graph is None:
            self.capture()
        self.graph.replay()

    def results(self):
        """Host arrays (harmonica units), one per problem, in input order."""
        self.torch.cuda.synchronize(self.device)
        return [o.cpu().numpy().reshape(s) for o, s in zip(self.outputs, self.shapes)]

    def singular(self):
        """Per-problem flags: a point lies on a singular point of a prism."""
        return self.flags.cpu().numpy()[: len(self.fields)].astype(bool)

    def close(self):
        if getattr(self, "handle", None):
            self.lib.hg_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001 - interpreter shutdown
            pass


def prism_gravity_batch(problems, chunk_prisms=0, n_ctas=0, disable_checks=False, device=None,
                        shapes="auto"):
    """
    Forward many problems in one persistent launch; returns a list of arrays
    equal (within FP64 rounding) to ``prism_gravity`` of each problem.  The
    work shape per field is autotuned by default (see :class:`PrismBatch`).
    """
    batch = PrismBatch(problems, chunk_prisms, n_ctas, check_singular=not disable_checks,
                       device=device, validate=not disable_checks, shapes=shapes)
    try:
        batch.run()
        results = batch.results()
        if not disable_checks and batch.singular().any():
            warnings.warn("Found observation point on singular point of a prism.",
                          UserWarning, stacklevel=2)
        return results
    finally:
        batch.close()


# ----------------------------------------------------------------------
# autotuner

def signature(problems):
    """Coarse key of a problem set: count, log2 of total pairs, field mix."""
    pairs = sum(np.size(p["coordinates"][0]) * np.shape(p["prisms"])[0] for p in problems)
    fields = sorted({p["field"] for p in problems})
    return f"n{len(problems)}-p{int(np.log2(max(pairs, 1)))}-{'+'.join(fields)}"


def _load_cache(path):
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _time_batch(problems, shapes, repeats, dev):
    """Best of ``repeats`` timed runs (ms, CUDA events) after one warm-up."""
    import torch

    b = PrismBatch(problems, device=dev, validate=False, shapes=shapes)  # None: fixed plan
    try:
        b.run()
        torch.cuda.synchronize(dev)
        best = float("inf")
        for _ in range(repeats):
            t0 = torch.cuda.Event(enable_timing=True)
            t1 = torch.cuda.Event(enable_timing=True)
            t0.record()
            b.run()
            t1.record()
            torch.cuda.synchronize(dev)
            best = min(best, t0.elapsed_time(t1))
        return best, b.info()["ctas"]
    finally:
        b.close()


def autotune(problems, chunks=(2048, 8192, 32768), points_per_cta=(64, 128),
             cta_multipliers=(1, 2), repeats=1, cache=DEFAULT_CACHE, device=None, sample=8):
    """
    Pick, per field of a problem set, the work shape by timing candidates.

    For each field present, an evenly strided sample of at most ``sample`` of
    its problems is run with every combination of points per CTA (the point
    tile of a work item and the prism tile staged in shared memory), prisms
    per work item and persistent CTAs (``cta_multipliers`` x the occupancy
    of one wave, divided by the largest multiplier), ``repeats`` timed runs
    after one warm-up (CUDA events), and against the fixed shape (128 points
    per CTA, automatic chunk and CTAs).  The fastest shape per field is
    returned and cached under ``(device name, signature(problems))``::

        {"shapes": {field: {"chunk_prisms", "points_per_cta", "n_ctas", "ms",
                            "fixed_ms", "gain"}},
         "candidates": [...]}
    """
    import torch

    from .gravity import _device

    dev = _device(device)
    key = torch.cuda.get_device_name(dev) + "|" + signature(problems)
    key = hashlib.sha1(key.encode()).hexdigest()[:16] + "|" + key
    table = _load_cache(cache) if cache else {}
    if key in table:
        return table[key]
    fields = sorted({p["field"] for p in problems}, key=lambda f: FIELD_CODES[f])
    result = {"shapes": {}, "candidates": []}
    for field in fields:
        mine = [p for p in problems if p["field"] == field]
        if sample and len(mine) > sample:
            step = len(mine) / sample
            mine = [mine[int(k * step)] for k in range(sample)]
        fixed_ms, occ = _time_batch(mine, None, repeats, dev)
        best = None
        for ppc in points_per_cta:
            for chunk in chunks:
                for mult in cta_multipliers:
                    ctas = max(1, occ * (128 // ppc) * mult // max(cta_multipliers))
                    shape = {"chunk_prisms": int(chunk), "points_per_cta": int(ppc),
                             "n_ctas": int(ctas)}
                    ms, _ = _time_batch(mine, {field: shape}, repeats, dev)
                    result["candidates"].append({"field": field, **shape, "ms": ms})
                    if best is None or ms < best["ms"]:
                        best = {**shape, "ms": ms}
        best.update(fixed_ms=fixed_ms, gain=fixed_ms / best["ms"])
        result["shapes"][field] = best
    if cache:
        table[key] = result
        os.makedirs(os.path.dirname(cache), exist_ok=True)
        tmp = f"{cache}.{os.getpid()}.tmp"  # one writer per file; the rename is atomic
        with open(tmp, "w") as f:
            json.dump(table, f, indent=1)
        os.replace(tmp, cache)
    return result
