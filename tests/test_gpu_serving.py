"""The batched and serving forms on the GPU: every request's verdict and counts are the same
whether it runs alone, in a batch, or through the request queue mixed with other requests; a
cancelled batch reports its unfinished instances as cancelled; the queue rejects a request whose
initial reservation exceeds the whole pool, grows a running request's store from the pool, stops a
request at its per-request limit while others in the same server finish, rejects submissions once the
queue is full, reports a result once, and cancels running requests when it is destroyed."""
import ctypes

import pytest

from ptctcl_gb300 import capi, engine
from ptctcl_gb300.generator import config_instance
from test_gpu_parity import C4_SMALL, small_config3

pytestmark = pytest.mark.gpu

COUNTS = ("explored", "generated", "stored", "keys", "levels")


def _mix():
    items = [config_instance(4, s) for s in C4_SMALL]
    for seed in (0, 1, 3):
        items.append(small_config3(seed))
    return items


def test_server_matches_alone_and_batch():
    items = _mix()
    alone = [engine.batch_run([it]) for it in items]
    bv, bst = engine.batch_run(items)
    with engine.Server(budget_bytes=8 << 30, max_inflight=8) as srv:
        tickets = [srv.submit(*it) for it in items]
        srv.drain(timeout=600)
        got = [srv.poll(t) for t in tickets]
    for k, (it, (av, ast), g) in enumerate(zip(items, alone, got)):
        assert g is not None, k
        v, st = g
        assert st["status"] == capi.OK, (k, st["status"])
        assert v == av[0] == bv[k], (k, v, av[0], bv[k])
        for c in COUNTS:
            assert st[c] == ast[0][c] == bst[k][c], (k, c, st[c], ast[0][c], bst[k][c])


def test_batch_cancelled_before_start():
    items = [config_instance(4, s) for s in C4_SMALL[:4]]
    cancel = ctypes.c_int32(1)
    verdicts, stats = engine.batch_run(items, cancel=cancel)
    assert verdicts == [-1] * len(items)
    assert all(s["status"] == capi.E_CANCELLED for s in stats)


def test_batch_time_to_verdict_within_run():
    items = [config_instance(4, s) for s in C4_SMALL]
    _, stats = engine.batch_run(items)
    for s in stats:
        assert s["status"] == capi.OK
        assert 0.0 <= s["seconds"] <= stats[0]["device_seconds"] + 60.0


def test_server_rejects_over_budget():
    net, kind, p, q = config_instance(4, C4_SMALL[0])
    with engine.Server(budget_bytes=1024, max_inflight=2) as srv:
        with pytest.raises(capi.HoraError) as ei:
            srv.submit(net, kind, p, q)
        assert ei.value.code == capi.E_BUDGET


def test_batch_in_instance_chunks_matches_whole_levels():
    """A 1-byte successor budget runs every level of the batch one instance at a time; verdicts and
    counts stay those of the unchunked run."""
    import json
    import os
    import subprocess
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    code = ("import json, sys; sys.path.insert(0, %r); sys.path.insert(0, %r)\n"
            "from test_gpu_serving import _mix\n"
            "from ptctcl_gb300 import engine\n"
            "v, st = engine.batch_run(_mix())\n"
            "print(json.dumps([v, [{k: s[k] for k in %r} for s in st]]))\n") % (
        os.path.dirname(here), here, COUNTS)
    out = {}
    for budget in ("", "1"):
        env = dict(os.environ)
        env.pop("HORA_GB_SUCC_BUDGET", None)
        if budget:
            env["HORA_GB_SUCC_BUDGET"] = budget
        r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, r.stderr[-2000:]
        out[budget] = json.loads(r.stdout.strip().splitlines()[-1])
    assert out[""] == out["1"]


def test_server_result_reported_once():
    net, kind, p, q = config_instance(4, C4_SMALL[0])
    with engine.Server(budget_bytes=1 << 30, max_inflight=2) as srv:
        t = srv.submit(net, kind, p, q)
        srv.drain(timeout=120)
        assert srv.poll(t) is not None
        with pytest.raises(capi.HoraError) as ei:
            srv.poll(t)                       # released after the first report
        assert ei.value.code == capi.E_INVALID


def test_server_store_grows_from_the_pool():
    """A request whose store outgrows its initial reservation takes more from the pool and gets the
    verdict and counts of the batched form; with a pool barely larger than one reservation it stops
    with HORA_E_BUDGET instead."""
    net, kind, p, q = config_instance(2, 23)          # about 2e5 successors
    (bv,), (bst,) = engine.batch_run([(net, kind, p, q)])
    with engine.Server(budget_bytes=2 << 30, max_inflight=16) as srv:   # reservation: 2 GB / 64
        t = srv.submit(net, kind, p, q)
        srv.drain(timeout=300)
        v, st = srv.poll(t)
    assert st["status"] == capi.OK and v == bv
    for c in COUNTS:
        assert st[c] == bst[c], c
    big, bk, bp, bq = config_instance(2, 2483)        # 1.45M stored zones, far past 64 Ki
    d = big.dim
    floor = (1 << 16) * (d * d * 4 + 32) * 2
    with engine.Server(budget_bytes=floor + floor // 2, max_inflight=1) as srv:
        t = srv.submit(big, bk, bp, bq)
        srv.drain(timeout=300)
        v, st = srv.poll(t)
    assert st["status"] == capi.E_BUDGET and v == -1


def test_server_per_request_limit_stops_only_the_large_request():
    """With a large pool but a per-request limit of a few reservations, the large request stops with
    HORA_E_BUDGET while a small request served beside it gets the batched form's verdict and
    counts."""
    small = config_instance(2, 23)
    (sv,), (sst,) = engine.batch_run([small])
    big = config_instance(2, 2483)                   # 1.45M stored zones
    d = big[0].dim
    floor = (1 << 16) * (d * d * 4 + 32) * 2
    with engine.Server(budget_bytes=16 << 30, max_inflight=4, per_request_bytes=4 * floor) as srv:
        tb = srv.submit(*big)
        ts = srv.submit(*small)
        srv.drain(timeout=300)
        bv, bst = srv.poll(tb)
        v, st = srv.poll(ts)
    assert bst["status"] == capi.E_BUDGET and bv == -1
    assert st["status"] == capi.OK and v == sv
    for c in COUNTS:
        assert st[c] == sst[c], c


def test_server_rejects_when_the_queue_is_full():
    """One slot, at most one waiting request: of five submissions made while a long request runs, at
    most two are accepted (the running one and one waiting) and the rest are rejected at once."""
    import time
    big = config_instance(3, 0)                      # runs for seconds
    srv = engine.Server(budget_bytes=8 << 30, max_inflight=1, max_queued=1)
    try:
        accepted, rejected = 0, 0
        for _ in range(5):
            try:
                srv.submit(*big)
                accepted += 1
            except capi.HoraError as e:
                assert e.code == capi.E_BUDGET
                rejected += 1
        assert 1 <= accepted <= 2 and rejected == 5 - accepted
        t = time.perf_counter()
    finally:
        srv.close()
    assert time.perf_counter() - t < 10.0


def test_server_destroy_cancels_running_requests():
    import time
    big, bk, bp, bq = config_instance(3, 0)            # phase 1 alone holds millions of zones
    srv = engine.Server(budget_bytes=64 << 30, max_inflight=2)
    srv.submit(big, bk, bp, bq)
    time.sleep(0.3)
    t = time.perf_counter()
    srv.close()
    assert time.perf_counter() - t < 10.0
