"""
Failure handling of the serving loop's host logic (PrismServer), on CPU:
cancelled requests, rejected admission, a failed device allocation, a
scheduler exception and a close without draining.  The admission and
scheduler code under test is the server's own; only the device upload is
replaced by CPU tensors (no kernel runs), so no GPU is needed and no GPU
fault is involved.
"""

import collections
import queue
import threading
from types import SimpleNamespace

import numpy as np
import pytest
import torch

from harmonica_gb300 import _native
from harmonica_gb300.serve import PrismServer


class _Event:
    def record(self, stream=None):
        pass


def _skeleton(budget=1e9, max_active=4):
    """A PrismServer without its device state or scheduler thread."""
    srv = PrismServer.__new__(PrismServer)
    srv.torch = SimpleNamespace(cuda=SimpleNamespace(Event=_Event))
    srv.dev = None
    srv.copy = None
    srv.budget = float(budget)
    srv.used = 0.0
    srv.round_pairs = 1e6
    srv.rounds_in_flight = 2
    srv.max_active = max_active
    srv.max_chunk = 2048
    srv.layers = collections.OrderedDict()
    srv.inbox = queue.Queue()
    srv.pending = collections.deque()
    srv.active = {}
    srv.free_slots = list(range(max_active - 1, -1, -1))
    srv.in_flight = collections.deque()
    srv.completed = []
    srv.errors = []
    srv.rounds = 0
    srv.pairs_done = 0.0
    srv._ids = 0
    srv._lock = threading.RLock()
    srv._stop = threading.Event()
    srv._broken = None
    srv.nominal_rate = 1e10
    srv.max_backlog_s = None
    srv.rates = {code: 1e10 for code in range(10)}
    srv.backlog_s = 0.0
    srv.rejected = 0
    srv.table = (_native.HgProblemPlan * max_active)()
    srv.flags = torch.zeros(max_active, dtype=torch.int32)
    srv.uploads = []

    def upload(req, layer, n_chunks):
        srv.uploads.append(req.id)
        points = [torch.zeros(max(req.n_obs, 1), dtype=torch.float64) for _ in range(3)]
        n_prisms = layer.n_prisms if layer is not None else req.n_prisms
        soa = torch.zeros((7, max(n_prisms, 1)), dtype=torch.float64)
        out = torch.zeros(max(req.n_obs, 1), dtype=torch.float64)
        part = torch.zeros(max(req.n_obs * n_chunks, 1), dtype=torch.float64)
        pinned = torch.zeros(max(req.n_obs, 1), dtype=torch.float64)
        return points + [soa, out, part], n_prisms, pinned

    srv._upload = upload
    return srv


def _problem(n_obs=10, n_prisms=3):
    rng = np.random.default_rng(n_obs + n_prisms)
    coords = (rng.uniform(0, 100, n_obs), rng.uniform(0, 100, n_obs), np.full(n_obs, 10.0))
    w = rng.uniform(0, 90, n_prisms)
    s = rng.uniform(0, 90, n_prisms)
    prisms = np.column_stack([w, w + 5, s, s + 5, np.full(n_prisms, -20.0),
                              np.full(n_prisms, -5.0)])
    return coords, prisms, np.full(n_prisms, 2670.0)


def _submit(srv, **kw):
    coords, prisms, density = _problem(**kw)
    fut = srv.submit(coords, "g_z", prisms=prisms, density=density)
    srv.pending.append(srv.inbox.get_nowait())
    return fut


def test_cancelled_while_waiting_is_skipped():
    srv = _skeleton()
    first = _submit(srv)
    second = _submit(srv)
    assert first.cancel()
    srv._admit()
    assert first.cancelled()
    assert srv.uploads == [1]  # only the second request reached the device
    assert 1 in srv.active and 0 not in srv.active
    # admitted requests run to completion: their futures can no longer be cancelled
    assert not second.cancel() and second.running()


def test_rejections_fail_only_their_request():
    srv = _skeleton(budget=50_000)
    unknown = srv.submit(_problem()[0], "g_z", layer="nope")
    srv.pending.append(srv.inbox.get_nowait())
    big = _submit(srv, n_obs=2000, n_prisms=3)  # 2000 x 8 B x 5 rows > budget
    ok = _submit(srv)
    srv._admit()
    with pytest.raises(KeyError):
        unknown.result(0)
    with pytest.raises(MemoryError):
        big.result(0)
    (admitted,) = srv.active
    assert ok.running() and srv.uploads == [admitted]


def test_failed_allocation_fails_that_request_and_serving_goes_on():
    srv = _skeleton()
    upload = srv._upload

    def failing_once(req, layer, n_chunks):
        if req.id == 0:
            raise RuntimeError("CUDA out of memory (simulated)")
        return upload(req, layer, n_chunks)

    srv._upload = failing_once
    first = _submit(srv)
    second = _submit(srv)
    srv._admit()
    with pytest.raises(RuntimeError, match="simulated"):
        first.result(0)
    # nothing of the failed request stays on the books
    assert list(srv.active) == [1]
    assert srv.used == pytest.approx(srv.active[1].bytes)
    assert sorted(srv.free_slots + [srv.active[1].slot]) == list(range(srv.max_active))
    assert second.running()


def test_failed_allocation_against_a_resident_layer_keeps_it_idle():
    srv = _skeleton()
    layer = SimpleNamespace(key="topo", n_prisms=5, users=0, last_used=0.0, bytes=7 * 5 * 8,
                            soa=torch.zeros((7, 5), dtype=torch.float64))
    srv.layers["topo"] = layer

    def failing(req, layer, n_chunks):
        raise RuntimeError("pinned allocation failed (simulated)")

    srv._upload = failing
    fut = srv.submit(_problem()[0], "g_z", layer="topo")
    srv.pending.append(srv.inbox.get_nowait())
    srv._admit()
    with pytest.raises(RuntimeError, match="simulated"):
        fut.result(0)
    assert layer.users == 0 and srv.used == 0.0  # still evictable


def test_empty_request_completes_with_zeros():
    srv = _skeleton()
    fut = _submit(srv, n_obs=4, n_prisms=0)
    srv._admit()
    np.testing.assert_array_equal(fut.result(0), np.zeros(4))
    assert srv.used == 0.0 and not srv.active


def test_scheduler_exception_fails_every_waiting_request():
    srv = _skeleton()
    waiting = [_submit(srv) for _ in range(2)]
    coords, prisms, density = _problem()
    queued = srv.submit(coords, "g_z", prisms=prisms, density=density)  # still in the inbox

    def broken_admit():
        raise RuntimeError("scheduler fault (simulated)")

    srv._admit = broken_admit
    with pytest.raises(RuntimeError, match="simulated"):
        srv._run()
    for fut in waiting + [queued]:
        with pytest.raises(RuntimeError, match="simulated"):
            fut.result(0)
    assert len(srv.errors) == 1
    # a stopped server refuses new work instead of leaving its future unresolved
    with pytest.raises(RuntimeError, match="stopped after an error"):
        srv.submit(coords, "g_z", prisms=prisms, density=density)


def test_close_without_drain_fails_unfinished_requests():
    srv = _skeleton()
    waiting = [_submit(srv) for _ in range(3)]
    srv._admit = lambda: None  # nothing is admitted before the close
    srv._drain = False
    srv._stop.set()
    srv._run()
    for fut in waiting:
        with pytest.raises(RuntimeError, match="closed before this request finished"):
            fut.result(0)
    coords, prisms, density = _problem()
    with pytest.raises(RuntimeError, match="closed"):
        srv.submit(coords, "g_z", prisms=prisms, density=density)


def test_close_with_drain_serves_requests_still_in_the_inbox():
    """A drained close does not stop while requests sit in the inbox."""
    srv = _skeleton()
    coords, prisms, density = _problem(n_obs=3, n_prisms=0)
    fut = srv.submit(coords, "g_z", prisms=prisms, density=density)
    srv._drain = True
    srv._stop.set()
    srv._run()  # empty request: admitted and completed without any round
    np.testing.assert_array_equal(fut.result(0), np.zeros(3))


def test_metrics_text_parses_as_prometheus_exposition():
    srv = _skeleton()
    for k, latency in enumerate([0.1, 0.2, 0.3, 0.4]):
        srv.completed.append(SimpleNamespace(t_submit=10.0 * k, t_done=10.0 * k + latency))
    srv.rounds, srv.pairs_done, srv.used = 3, 1.5e9, 4096.0
    _submit(srv)  # one request waiting for admission
    text = srv.metrics_text()
    parser = pytest.importorskip("prometheus_client.parser")
    families = {f.name: f for f in parser.text_string_to_metric_families(text)}
    value = {f.name: f.samples[0].value for f in families.values() if f.type != "summary"}
    assert value["hg_server_requests_completed"] == 4
    assert value["hg_server_requests_waiting"] == 1
    assert value["hg_server_rounds"] == 3
    assert value["hg_server_pairs"] == 1.5e9
    assert value["hg_server_device_bytes"] == 4096.0
    latency = {s.name + s.labels.get("quantile", ""): s.value
               for s in families["hg_server_latency_seconds"].samples}
    assert latency["hg_server_latency_seconds0.5"] == pytest.approx(0.25)
    assert latency["hg_server_latency_seconds_count"] == 4
    assert latency["hg_server_latency_seconds_sum"] == pytest.approx(1.0)


def _layer(key, n_prisms):
    from harmonica_gb300.serve import _Layer

    return _Layer(key, torch.zeros((7, n_prisms), dtype=torch.float64), n_prisms)


def test_reregistering_a_layer_releases_the_old_bytes():
    srv = _skeleton()
    srv._add_layer(_layer("topo", 100))
    assert srv.used == 7 * 100 * 8
    srv._add_layer(_layer("topo", 40))  # replaced: the old 100 prisms are released
    assert srv.used == 7 * 40 * 8 and srv.layers["topo"].n_prisms == 40
    assert srv.unregister_layer("topo") == 7 * 40 * 8
    assert srv.used == 0.0 and not srv.layers
    with pytest.raises(KeyError):
        srv.unregister_layer("topo")


def test_a_layer_in_use_is_neither_replaced_nor_dropped():
    srv = _skeleton()
    srv._add_layer(_layer("topo", 10))
    fut = srv.submit(_problem()[0], "g_z", layer="topo")
    srv.pending.append(srv.inbox.get_nowait())
    srv._admit()
    assert fut.running() and srv.layers["topo"].users == 1
    with pytest.raises(RuntimeError, match="in use"):
        srv._add_layer(_layer("topo", 20))
    with pytest.raises(RuntimeError, match="in use"):
        srv.unregister_layer("topo")
    assert srv.layers["topo"].n_prisms == 10


def test_earliest_virtual_deadline_first_lets_no_request_starve():
    """Rounds take items earliest virtual deadline first (arrival + pairs at
    the nominal rate): a small request that arrives after a large one goes
    first while its deadline is earlier, and the large one's turn comes as
    soon as its deadline is the earliest, however many small requests follow."""
    srv = _skeleton(max_active=8)
    srv.nominal_rate = 1e3  # pairs/s: deadlines far apart for these small cases
    srv.round_pairs = 1  # one work item per round
    big = _submit(srv, n_obs=300, n_prisms=3)    # 900 pairs: deadline t0 + 0.9 s
    small = _submit(srv, n_obs=10, n_prisms=3)   # 30 pairs: deadline t1 + 0.03 s
    srv._admit()
    reqs = {r.n_obs: r for r in srv.active.values()}
    assert reqs[10].deadline < reqs[300].deadline
    items, _, finishing, _ = srv._plan_round()
    assert items[0, 0] == reqs[10].slot and finishing == [reqs[10]]
    # a later small request whose deadline falls after the big one's waits
    reqs[300].deadline = reqs[10].deadline - 1.0  # the big request has aged past it
    late = _submit(srv, n_obs=10, n_prisms=3)
    srv._admit()
    items, _, _, _ = srv._plan_round()
    assert items[0, 0] == reqs[300].slot
    assert big.running() and small.running() and late.running()


def test_load_shedding_refuses_requests_beyond_the_backlog_and_counts_them():
    """Work is priced per field at its measured rate: a request is refused
    when the backlog plus its own work exceeds max_backlog_s."""
    from harmonica_gb300.serve import ServerOverloaded

    srv = _skeleton()
    srv.max_backlog_s = 1.0
    srv.rates[3] = 1000.0  # g_z pairs/s
    srv.rates[0] = 250.0   # potential: four times the cost per pair
    first = _submit(srv, n_obs=200, n_prisms=3)  # 600 g_z pairs: 0.6 s of work
    assert srv.backlog_s == pytest.approx(0.6)
    coords, prisms, density = _problem(n_obs=200, n_prisms=3)
    refused = srv.submit(coords, "g_z", prisms=prisms, density=density)  # 1.2 s > 1 s
    with pytest.raises(ServerOverloaded, match="backlog"):
        refused.result(0)
    assert srv.rejected == 1 and srv.inbox.empty()
    assert srv.backlog_s == pytest.approx(0.6)
    coords, prisms, density = _problem(n_obs=40, n_prisms=3)  # 120 pairs of potential: 0.48 s
    too_costly = srv.submit(coords, "potential", prisms=prisms, density=density)
    with pytest.raises(ServerOverloaded):
        too_costly.result(0)
    fits = _submit(srv, n_obs=100, n_prisms=3)  # 0.3 s of g_z with the first: accepted
    assert srv.backlog_s == pytest.approx(0.9)
    # a finished or failed request leaves the backlog
    first.set_running_or_notify_cancel()
    first.set_result(np.zeros(200))
    assert srv.backlog_s == pytest.approx(0.3)
    assert fits.cancel() and srv.backlog_s == pytest.approx(0.0)
    assert srv.stats()["rejected"] == 2
