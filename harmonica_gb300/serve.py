"""
Serving loop with continuous batching for prism forward solves on one GPU.

Requests (observation points + a prism layer or prism list + one field)
arrive at any time through :meth:`PrismServer.submit` and get a
``concurrent.futures.Future``.  A scheduler thread:

* **admits** queued requests in arrival order while their device memory
  (points, output, partial sums, and the prisms unless they are a resident
  layer) fits the memory budget, copying their inputs on a copy stream while
  the GPU computes;
* keeps **resident layers** (:meth:`register_layer`) on the device so repeated
  requests against the same model skip the upload; idle layers are evicted
  least-recently-used when memory is needed;
* launches **rounds**: each round is one persistent launch (``hg_round_run``)
  over work items (request, 128-point tile, prism chunk) taken from every
  admitted request, earliest virtual deadline first (arrival time plus the
  request's pairs at the nominal rate: small requests overtake large ones,
  and a large request's turn comes once its deadline is the earliest, so
  none starves), up to a per-round budget of point-prism pairs, so requests
  that arrive while others are on the GPU join the next round instead of
  waiting for the earlier ones to finish;
* optionally **sheds load** (``max_backlog_s``): a request is refused at
  submission (its future fails with :class:`ServerOverloaded`) when the
  unfinished work, its own included, would take longer than that; work is
  priced per field at the pairs/s measured on the GPU (each round times
  each field's launch with CUDA events), so the latency of the accepted
  requests stays bounded under overload;
* finishes requests with ``hg_round_reduce`` (each point's chunks added in
  fixed order), copies results to pinned host memory and resolves the
  futures, recording arrival-to-result latency.

Work items of a request are cut with a chunk size that depends only on that
request, and its chunks are reduced in fixed order, so a result is bitwise
the same whether the request ran alone or mixed with others.

This replaces calling ``harmonica.prism_gravity``
(``src/harmonica/_forward/prisms/gravity.py:51-236``) once per request.
"""

import collections
import ctypes
import queue
import threading
import time
from concurrent.futures import Future, InvalidStateError

import numpy as np

from . import _native
from ._trace import stage
from .fields import FIELD_CODES, TENSOR_FIELDS
from .gravity import _prepare, pack_prisms

KTHREADS = 128  # points per work item (the kernels' tile)


# Weight of a pair of each field relative to g_z: the virtual deadlines of
# the scheduling order and the prior of the per-field rates until each
# field's launches have been timed (the other first derivatives as g_z, the
# other tensor components as g_zz).  The values are the layer kernels'
# relative costs on GB300 when the served stream was tuned (g_z 1.21e10,
# potential 3.41e9, g_zz 2.39e10 pairs/s).  The current kernels' ratios
# (potential 2.76, g_zz 0.59) gave served / plain 1.026 on that stream, these
# 1.03-1.04 over three runs, so these stay.
FIELD_COST = {"potential": 3.55, "g_e": 1.0, "g_n": 1.0, "g_z": 1.0, "g_ee": 0.5, "g_nn": 0.5,
              "g_zz": 0.5, "g_en": 0.5, "g_ez": 0.5, "g_nz": 0.5}


class ServerOverloaded(RuntimeError):
    """A request refused at submission because the server's backlog would
    exceed its ``max_backlog_s``."""


def chunk_for(n_prisms, max_chunk=2048):
    """Prism chunk of a request: a function of the request alone, in whole
    128-prism tiles (the cap is rounded down to a whole tile)."""
    cap = max(128, (int(max_chunk) // 128) * 128)
    return max(128, min(cap, ((n_prisms + 127) // 128) * 128))


def _fail(req, exc):
    """Resolve a request's future with ``exc`` unless it is already done
    (finished, failed or cancelled by its caller)."""
    if not req.future.done():
        try:
            req.future.set_exception(exc)
        except InvalidStateError:  # cancelled between the check and the call
            pass


class _Layer:
    __slots__ = ("key", "soa", "n_prisms", "bytes", "users", "last_used")

    def __init__(self, key, soa, n_prisms):
        self.key = key
        self.soa = soa
        self.n_prisms = n_prisms
        self.bytes = soa.numel() * 8
        self.users = 0
        self.last_used = time.perf_counter()


class _Request:
    def __init__(self, rid, coords, field, layer_key, prisms, density, check_singular):
        self.id = rid
        self.coords = coords
        self.field = field
        self.layer_key = layer_key
        self.prisms = prisms
        self.density = density
        self.check_singular = check_singular
        self.future = Future()
        self.t_submit = time.perf_counter()
        self.t_done = None
        self.slot = -1
        self.layer = None
        self.tensors = []
        self.bytes = 0
        self.n_obs = coords[0].size
        self.n_prisms = prisms.shape[0] if prisms is not None else None
        self.pairs = 0.0      # point-prism pairs of the request
        self.deadline = 0.0   # virtual deadline: arrival + pairs / nominal rate
        self.next_item = 0
        self.n_items = 0
        self.chunk = 0
        self.n_chunks = 0
        self.pinned_out = None
        self.shape = None


class PrismServer:
    """
    Continuous-batching server for prism forward solves on one GPU.

    Parameters
    ----------
    memory_budget : float
        Device bytes the server may hold for admitted requests and resident
        layers (admission stops when the next request would not fit).
    round_pairs : float
        Target point-prism pairs per round (a round is one persistent launch
        per field).
    max_active : int
        Size of the device problem table (admitted requests at once).
    chunk : int
        Largest prism chunk of a work item.  A work item (128 points x the
        chunk) runs on one CTA, so the last items of a launch leave SMs idle
        for up to one item's time: the defaults (1.6e9-pair rounds of
        128 x 512 items) keep each field's launch many items deep.  Measured
        on the served stream of a GB300 (Poisson 200 req/s, g_z / potential /
        g_zz): 4e8-pair rounds of 2048-prism items 7.5e9 pairs/s; 4e8 and 512
        1.13e10; 1.6e9 and 2048 1.17e10; 1.6e9 and 512 1.24e10.
    nominal_rate : float
        g_z pairs per second; with the relative costs of ``FIELD_COST`` it
        gives the work of a request for the virtual deadlines of the
        scheduling order and the first estimate of each field's rate for
        load shedding (then replaced by the field's measured rate).
    max_backlog_s : float or None
        Refuse new requests (:class:`ServerOverloaded`) while the unfinished
        work, the new request's included, exceeds this many seconds at the
        measured rates; ``None`` accepts everything.
    """

    def __init__(self, device=None, memory_budget=120e9, round_pairs=1.6e9, max_active=1024,
                 chunk=512, n_ctas=0, rounds_in_flight=2, nominal_rate=1e10,
                 max_backlog_s=None):
        import torch

        from .gravity import _device

        self.torch = torch
        self.dev = _device(device)
        self.lib = _native.lib()
        self.budget = float(memory_budget)
        self.used = 0.0
        self.round_pairs = float(round_pairs)
        self.max_active = int(max_active)
        self.max_chunk = int(chunk)
        self.n_ctas = int(n_ctas)
        self.rounds_in_flight = int(rounds_in_flight)
        self.nominal_rate = float(nominal_rate)
        self.max_backlog_s = None if max_backlog_s is None else float(max_backlog_s)
        # measured pairs/s of each field's launches (field code -> rate)
        self.rates = {code: float(nominal_rate) / FIELD_COST[name]
                      for name, code in FIELD_CODES.items()}
        self.backlog_s = 0.0  # estimated seconds of accepted, unfinished work
        self.rejected = 0
        self.layers = collections.OrderedDict()
        self.inbox = queue.Queue()
        self.pending = collections.deque()
        self.active = {}
        self.free_slots = list(range(self.max_active - 1, -1, -1))
        self.in_flight = collections.deque()
        self.completed = []
        self.errors = []
        self.rounds = 0
        self.pairs_done = 0.0
        self._ids = 0
        self._lock = threading.RLock()  # re-entered by future callbacks run under it
        self._stop = threading.Event()
        self._broken = None  # the exception that stopped the scheduler, if any
        with torch.cuda.device(self.dev):
            self.compute = torch.cuda.Stream(self.dev)
            self.copy = torch.cuda.Stream(self.dev)
            self.table_dev = torch.empty(self.max_active * ctypes.sizeof(_native.HgProblemPlan),
                                         dtype=torch.uint8, device=self.dev)
            self.counter = torch.zeros(10, dtype=torch.int64,
                                       device=self.dev)  # one per field code
            self.flags = torch.zeros(self.max_active, dtype=torch.int32, device=self.dev)
        self.table = (_native.HgProblemPlan * self.max_active)()
        self._ring = [self._pinned_round_buffers() for _ in range(self.rounds_in_flight + 2)]
        self._ring_next = 0
        self.thread = threading.Thread(target=self._run, name="prism-server", daemon=True)
        self.thread.start()

    # ------------------------------------------------------------------ api
    def register_layer(self, key, prisms, density):
        """Keep a prism model resident (evictable when idle); returns its bytes.

        Registering an existing key replaces that layer when no admitted
        request uses it (``RuntimeError`` otherwise)."""
        with self._lock:
            self._check_replaceable(key)
        torch = self.torch
        _, _, p_np, d_np = _prepare(([0.0], [0.0], [0.0]), prisms, density, False)
        with torch.cuda.device(self.dev), torch.cuda.stream(self.copy):
            pr = torch.from_numpy(np.ascontiguousarray(p_np)).to(self.dev, non_blocking=False)
            rho = torch.from_numpy(np.ascontiguousarray(d_np)).to(self.dev, non_blocking=False)
            soa = pack_prisms(pr, rho)
            self.copy.synchronize()
        layer = _Layer(key, soa, p_np.shape[0])
        with self._lock:
            self._add_layer(layer)
        return layer.bytes

    def unregister_layer(self, key):
        """Drop a resident layer that no admitted request uses; returns the
        device bytes it held (``KeyError`` for an unknown key,
        ``RuntimeError`` while it is in use)."""
        with self._lock:
            layer = self.layers[key]
            self._check_replaceable(key)
            del self.layers[key]
            self.used -= layer.bytes
        return layer.bytes

    def _check_replaceable(self, key):
        old = self.layers.get(key)
        if old is not None and old.users:
            raise RuntimeError(f"layer {key!r} is in use by admitted requests")

    def _add_layer(self, layer):
        """Book a layer, replacing an idle one of the same key (its bytes
        are released)."""
        self._check_replaceable(layer.key)
        old = self.layers.pop(layer.key, None)
        if old is not None:
            self.used -= old.bytes
        self.layers[layer.key] = layer
        self.used += layer.bytes

    def submit(self, coordinates, field, layer=None, prisms=None, density=None,
               check_singular=False):
        """Queue one forward solve; returns a Future of the result array.

        The future may be cancelled while the request waits for admission;
        once admitted it runs to completion.  Raises ``RuntimeError`` after
        :meth:`close` or after the scheduler stopped on an error."""
        self._check_open()
        if field not in FIELD_CODES:
            raise ValueError(f"Gravitational field {field} not recognized")
        cast, coords, p_np, d_np = _prepare(
            coordinates,
            prisms if prisms is not None else np.zeros((0, 6)),
            density if density is not None else np.zeros(0),
            prisms is None,
        )
        if layer is None and prisms is None:
            raise ValueError("submit needs a registered layer key or prisms and density")
        req = _Request(-1, coords, field, layer, p_np if layer is None else None,
                       d_np if layer is None else None,
                       check_singular and field in TENSOR_FIELDS)
        req.shape = cast.shape
        with self._lock:
            known = self.layers.get(layer) if layer is not None else None
            n_prisms = known.n_prisms if known is not None else (req.n_prisms or 0)
            req.pairs = float(req.n_obs) * float(n_prisms)
            req.deadline = req.t_submit + req.pairs * FIELD_COST[field] / self.nominal_rate
            req.cost_s = req.pairs / self.rates[FIELD_CODES[field]]
            if (self.max_backlog_s is not None and self.backlog_s > 0
                    and self.backlog_s + req.cost_s > self.max_backlog_s):
                self.rejected += 1
                req.future.set_exception(ServerOverloaded(
                    f"request of {req.pairs:.3g} pairs ({req.cost_s:.2f} s of work) refused: "
                    f"the backlog is {self.backlog_s:.2f} s of work (limit "
                    f"{self.max_backlog_s} s)"))
                return req.future
            req.id = self._ids
            self._ids += 1
            self.backlog_s += req.cost_s
        req.future.add_done_callback(self._forget_backlog(req))
        self.inbox.put(req)
        if self._broken is not None:  # the scheduler stopped while this was queued
            _fail(req, RuntimeError("the prism server stopped after an error"))
        return req.future

    def _forget_backlog(self, req):
        """Callback for a request's future: its work leaves the backlog when
        it finishes, fails or is cancelled."""

        def done(_future):
            with self._lock:
                self.backlog_s = max(0.0, self.backlog_s - req.cost_s)

        return done

    def _check_open(self):
        if self._broken is not None:
            raise RuntimeError("the prism server stopped after an error") from self._broken
        if self._stop.is_set():
            raise RuntimeError("the prism server is closed")

    def close(self, drain=True, timeout=None):
        """Stop the scheduler (after finishing queued work if ``drain``)."""
        self._drain = drain
        self._stop.set()
        self.thread.join(timeout)

    def stats(self):
        lat = np.array([r.t_done - r.t_submit for r in self.completed])
        out = {"completed": len(self.completed), "rounds": self.rounds,
               "pairs_done": self.pairs_done, "errors": len(self.errors),
               "rejected": self.rejected,
               "rates_pairs_per_s": {name: self.rates[code] for name, code in FIELD_CODES.items()}}
        if lat.size:
            out.update(p50_ms=float(np.percentile(lat, 50) * 1e3),
                       p99_ms=float(np.percentile(lat, 99) * 1e3),
                       mean_ms=float(lat.mean() * 1e3))
        return out

    def metrics_text(self, prefix="hg_server"):
        """The server's counters in the Prometheus text exposition format,
        for a scrape endpoint: requests completed, admitted and waiting,
        rounds, point-prism pairs done, device bytes held, scheduler errors
        and the arrival-to-result latency quantiles (seconds)."""
        st = self.stats()
        with self._lock:
            waiting = len(self.pending) + self.inbox.qsize()
            active = len(self.active)
            used = self.used
        rows = [
            ("requests_completed_total", "counter", "Requests finished with a result",
             st["completed"]),
            ("requests_active", "gauge", "Requests admitted to the device", active),
            ("requests_waiting", "gauge", "Requests waiting for admission", waiting),
            ("rounds_total", "counter", "Persistent launches issued", st["rounds"]),
            ("pairs_total", "counter", "Point-prism pairs of finished requests",
             st["pairs_done"]),
            ("device_bytes", "gauge", "Device bytes held by requests and layers", used),
            ("scheduler_errors_total", "counter", "Exceptions that stopped the scheduler",
             st["errors"]),
        ]
        lines = []
        for name, kind, text, value in rows:
            lines += [f"# HELP {prefix}_{name} {text}", f"# TYPE {prefix}_{name} {kind}",
                      f"{prefix}_{name} {float(value)!r}"]
        name = f"{prefix}_latency_seconds"
        lines += [f"# HELP {name} Arrival-to-result latency of finished requests",
                  f"# TYPE {name} summary"]
        for q, key in (("0.5", "p50_ms"), ("0.99", "p99_ms")):
            if key in st:
                lines.append(f'{name}{{quantile="{q}"}} {st[key] / 1e3!r}')
        total = st.get("mean_ms", 0.0) * st["completed"] / 1e3
        lines += [f"{name}_sum {total!r}", f"{name}_count {st['completed']}"]
        return "\n".join(lines) + "\n"

    # ----------------------------------------------------------- internals
    def _pinned_round_buffers(self):
        torch = self.torch
        return {
            "table": torch.empty(self.max_active * ctypes.sizeof(_native.HgProblemPlan),
                                 dtype=torch.uint8, pin_memory=True),
            "items": torch.empty(0, dtype=torch.int32, pin_memory=True),
            "ids": torch.empty(0, dtype=torch.int32, pin_memory=True),
            "event": None,
        }

    def _request_bytes(self, req, layer):
        chunk = chunk_for(layer.n_prisms if layer else req.n_prisms, self.max_chunk)
        n_prisms = layer.n_prisms if layer else req.n_prisms
        n_chunks = max(1, -(-n_prisms // chunk))
        b = 8 * req.n_obs * (3 + 1 + n_chunks)
        if layer is None:
            b += 8 * 7 * max(req.n_prisms, 1) + 8 * 7 * max(req.n_prisms, 1)
        return b, chunk, n_chunks

    def _evict_for(self, need):
        for key in list(self.layers):
            if self.used + need <= self.budget:
                return True
            layer = self.layers[key]
            if layer.users == 0:
                del self.layers[key]
                self.used -= layer.bytes
        return self.used + need <= self.budget

    def _admit(self):
        with self._lock:
            self._admit_locked()

    def _admit_locked(self):
        admitted = False
        while self.pending and self.free_slots:
            req = self.pending[0]
            if req.future.cancelled():  # cancelled by its caller while it waited
                self.pending.popleft()
                continue
            layer = None
            if req.layer_key is not None:
                layer = self.layers.get(req.layer_key)
                if layer is None:
                    self.pending.popleft()
                    _fail(req, KeyError(f"layer {req.layer_key!r} not registered"))
                    continue
            need, chunk, n_chunks = self._request_bytes(req, layer)
            if need > self.budget:
                self.pending.popleft()
                _fail(req, MemoryError(
                    f"request needs {need} device bytes, above the server budget"))
                continue
            if self.used + need > self.budget and not self._evict_for(need):
                break  # wait for memory to free up (arrival order is kept)
            self.pending.popleft()
            if not req.future.set_running_or_notify_cancel():
                continue  # cancelled just now; from here on it runs to completion
            try:
                tensors, n_prisms, pinned_out = self._upload(req, layer, n_chunks)
            except Exception as exc:  # noqa: BLE001 - an allocation or copy failed
                # this request fails alone: nothing of it is on the device
                # books yet, and the server keeps serving the others
                _fail(req, exc)
                continue
            if layer is not None:
                layer.users += 1
                layer.last_used = time.perf_counter()
                self.layers.move_to_end(layer.key)
            req.tensors += tensors
            e, n, u, soa, out, part = tensors[-6:]
            req.layer = layer
            req.bytes = need
            self.used += need
            if n_prisms == 0 or req.n_obs == 0:
                # nothing to sum: zeros (gravity.py:202 starts from np.zeros)
                req.t_done = time.perf_counter()
                if layer is not None:
                    layer.users -= 1
                self.used -= need
                req.tensors = []
                self.completed.append(req)
                req.future.set_result(np.zeros(req.shape))
                continue
            req.chunk = chunk
            req.n_chunks = -(-n_prisms // chunk) if n_prisms else 0
            req.n_items = -(-req.n_obs // KTHREADS) * req.n_chunks
            req.slot = self.free_slots.pop()
            req.pinned_out = pinned_out
            p = self.table[req.slot]
            p.obs_e, p.obs_n, p.obs_u = e.data_ptr(), n.data_ptr(), u.data_ptr()
            p.n_obs = req.n_obs
            p.prisms_soa = soa.data_ptr()
            p.prism_stride = soa.shape[1]
            p.n_prisms = n_prisms
            p.chunk = chunk
            p.n_chunks = req.n_chunks
            p.partials = part.data_ptr()
            p.out = out.data_ptr()
            p.singular_flag = self.flags[req.slot:].data_ptr()
            p.field = FIELD_CODES[req.field]
            p.check_singular = int(req.check_singular)
            self.active[req.id] = req
            admitted = True
        if admitted:
            self._copy_event = self.torch.cuda.Event()
            self._copy_event.record(self.copy)

    def _upload(self, req, layer, n_chunks):
        """Device copies of a request's points (and prisms, unless it uses a
        resident layer) and its output and partial-sum buffers, queued on the
        copy stream, and the pinned host buffer of its result.  Returns the
        device tensors (the output second to last), the number of prisms and
        the pinned buffer."""
        torch = self.torch
        tensors = []
        with torch.cuda.device(self.dev), torch.cuda.stream(self.copy):
            e, n, u = (torch.from_numpy(c).pin_memory().to(self.dev, non_blocking=True)
                       for c in req.coords)
            if layer is None:
                pr = torch.from_numpy(np.ascontiguousarray(req.prisms)).to(self.dev)
                rho = torch.from_numpy(np.ascontiguousarray(req.density)).to(self.dev)
                soa = pack_prisms(pr, rho) if req.n_prisms else torch.zeros(
                    (7, 1), dtype=torch.float64, device=self.dev)
                n_prisms = req.n_prisms
                tensors += [pr, rho]
            else:
                soa = layer.soa
                n_prisms = layer.n_prisms
            out = torch.empty(max(req.n_obs, 1), dtype=torch.float64, device=self.dev)
            part = torch.empty(max(req.n_obs * n_chunks, 1), dtype=torch.float64,
                               device=self.dev)
        pinned_out = torch.empty(max(req.n_obs, 1), dtype=torch.float64, pin_memory=True)
        return tensors + [e, n, u, soa, out, part], n_prisms, pinned_out

    def _plan_round(self):
        """Items for the next round: earliest virtual deadline first (ties in
        arrival order), then grouped by field (each field runs its own
        specialised persistent launch).  Returns (items, per-field item
        counts, finishing requests, per-field point-prism pairs)."""
        reqs = [r for r in self.active.values() if r.next_item < r.n_items]
        if not reqs:
            return None, None, [], None
        reqs.sort(key=lambda r: (r.deadline, r.id))
        budget = self.round_pairs
        parts, finishing = [], []
        pairs = np.zeros(10)
        for r in reqs:
            if budget <= 0:
                break
            per_item = KTHREADS * r.chunk
            take = int(min(r.n_items - r.next_item, max(1, budget // per_item)))
            k = np.arange(r.next_item, r.next_item + take, dtype=np.int64)
            items = np.empty((take, 4), dtype=np.int32)
            items[:, 0] = r.slot
            items[:, 1] = k // r.n_chunks  # tile
            items[:, 2] = k % r.n_chunks   # chunk
            items[:, 3] = 0
            n_prisms = r.layer.n_prisms if r.layer else r.n_prisms
            pts = np.minimum(KTHREADS, r.n_obs - items[:, 1].astype(np.int64) * KTHREADS)
            prs = np.minimum(r.chunk, n_prisms - items[:, 2].astype(np.int64) * r.chunk)
            pairs[FIELD_CODES[r.field]] += float(np.dot(pts, prs))
            parts.append((FIELD_CODES[r.field], items))
            r.next_item += take
            budget -= take * per_item
            if r.next_item == r.n_items:
                finishing.append(r)
        counts = np.zeros(10, dtype=np.int64)
        for code, items in parts:
            counts[code] += items.shape[0]
        order = sorted(range(len(parts)), key=lambda i: parts[i][0])  # stable
        return np.concatenate([parts[i][1] for i in order]), counts, finishing, pairs

    def _launch_round(self, items, counts, finishing, pairs):
        torch = self.torch
        buf = self._ring[self._ring_next]
        self._ring_next = (self._ring_next + 1) % len(self._ring)
        if buf["event"] is not None:
            buf["event"].synchronize()  # the previous use of this buffer has been consumed
        ctypes.memmove(buf["table"].data_ptr(), ctypes.addressof(self.table),
                       ctypes.sizeof(self.table))
        if buf["items"].numel() < items.size:
            buf["items"] = torch.empty(items.size * 2, dtype=torch.int32, pin_memory=True)
        buf["items"][: items.size].copy_(torch.from_numpy(items.ravel()))
        ids = np.array([r.slot for r in finishing], dtype=np.int32)
        if buf["ids"].numel() < ids.size:
            buf["ids"] = torch.empty(max(ids.size * 2, 16), dtype=torch.int32, pin_memory=True)
        if ids.size:
            buf["ids"][: ids.size].copy_(torch.from_numpy(ids))
        with torch.cuda.device(self.dev), torch.cuda.stream(self.compute):
            if getattr(self, "_copy_event", None) is not None:
                self.compute.wait_event(self._copy_event)
            self.table_dev.copy_(buf["table"], non_blocking=True)
            items_dev = buf["items"][: items.size].to(self.dev, non_blocking=True)
            stream = self.compute.cuda_stream
            # one launch per field, each between two events: the field's
            # measured rate prices its requests for load shedding
            timed, begin = [], 0
            for code in np.nonzero(counts)[0]:
                field_counts = (ctypes.c_int64 * 10)()
                field_counts[code] = int(counts[code])
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(self.compute)
                _native.check(self.lib.hg_round_run(
                    self.table_dev.data_ptr(), items_dev.data_ptr() + 16 * begin, field_counts,
                    self.n_ctas, self.counter.data_ptr(), stream))
                e1.record(self.compute)
                timed.append((int(code), float(pairs[code]), e0, e1))
                begin += int(counts[code])
            if ids.size:
                ids_dev = buf["ids"][: ids.size].to(self.dev, non_blocking=True)
                _native.check(self.lib.hg_round_reduce(self.table_dev.data_ptr(),
                                                       ids_dev.data_ptr(), ids.size, stream))
                for r in finishing:
                    out = r.tensors[-2]
                    r.pinned_out[: r.n_obs].copy_(out[: r.n_obs], non_blocking=True)
            ev = torch.cuda.Event()
            ev.record(self.compute)
        buf["event"] = ev
        self.in_flight.append((ev, finishing, timed))
        self.rounds += 1

    def _retire(self, block=False):
        while self.in_flight:
            ev, finishing, timed = self.in_flight[0]
            if not block and not ev.query():
                return
            ev.synchronize()
            self.in_flight.popleft()
            block = False
            now = time.perf_counter()
            self._measure_rates(timed)
            flags = None
            if any(r.check_singular for r in finishing):
                with self.torch.cuda.stream(self.compute):
                    flags = self.flags.cpu().numpy()
            for r in finishing:
                result = r.pinned_out[: r.n_obs].numpy().copy().reshape(r.shape)
                r.t_done = now
                self.pairs_done += float(r.n_obs) * float(
                    r.layer.n_prisms if r.layer else r.n_prisms)
                if flags is not None and flags[r.slot]:
                    r.future.singular = True
                with self._lock:
                    self._release(r)
                self.completed.append(r)
                r.future.set_result(result)

    def _measure_rates(self, timed):
        """Update each field's measured rate (pairs/s) from the finished
        round's launches (CUDA events around each), smoothed over rounds;
        launches shorter than a millisecond are too short to time."""
        for code, pairs, e0, e1 in timed:
            ms = e0.elapsed_time(e1)
            if pairs > 0 and ms >= 1.0:
                with self._lock:
                    self.rates[code] = 0.7 * self.rates[code] + 0.3 * pairs / (ms * 1e-3)

    def _release(self, r):
        self.active.pop(r.id, None)
        if r.layer is not None:
            r.layer.users -= 1
        self.used -= r.bytes
        with self.torch.cuda.stream(self.compute):
            self.flags[r.slot:r.slot + 1].zero_()
        self.free_slots.append(r.slot)
        r.tensors = []

    def _run(self):
        try:
            while True:
                idle = (not self.pending and not self.active and not self.in_flight
                        and self.inbox.empty())
                if self._stop.is_set() and (idle or not getattr(self, "_drain", True)):
                    break
                try:
                    req = self.inbox.get(timeout=0.002 if not idle else 0.05)
                    self.pending.append(req)
                    while True:
                        self.pending.append(self.inbox.get_nowait())
                except queue.Empty:
                    pass
                with stage("serve admit"):
                    self._admit()
                if len(self.in_flight) < self.rounds_in_flight:
                    items, counts, finishing, pairs = self._plan_round()
                    if items is not None:
                        with stage("serve round"):
                            self._launch_round(items, counts, finishing, pairs)
                        continue
                with stage("serve retire"):
                    self._retire(block=len(self.in_flight) >= self.rounds_in_flight)
        except Exception as exc:  # noqa: BLE001 - fail every waiting request
            self.errors.append(exc)
            self._broken = exc  # submit() refuses new work from here on
            self._fail_unfinished(exc)
            raise
        # closed without draining: requests still queued or on the device
        # will not finish (their device buffers stay referenced until the
        # server object goes away, as rounds may still be running)
        self._fail_unfinished(RuntimeError("the prism server was closed before this request "
                                           "finished"))

    def _fail_unfinished(self, exc):
        """Fail every request that has not finished: admitted, pending and
        still in the inbox."""
        while True:
            try:
                self.pending.append(self.inbox.get_nowait())
            except queue.Empty:
                break
        for r in list(self.active.values()) + list(self.pending):
            _fail(r, exc)
