"""Whole queries at the benchmark's full sizes against the oracle's verdict and counts, recorded by
tests/golden/make_full_size.py because the oracle needs minutes per query: config 2 (A[] not
deadlock, up to 1.45M stored zones and 20M successors) and config 3 (p --> q, violated by the early
witness after up to 110M successors). A second run must reproduce every count (the merge order is
canonical, not scheduling-dependent). Collected near the end (only the allocation-free entry
point's test comes after it), so that a failure here comes after the parity tests have run."""
import json
import os

import pytest

from ptctcl_gb300 import engine
from ptctcl_gb300.engine import Backend, ReachStats
from ptctcl_gb300.generator import config_instance

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROWS = json.load(open(os.path.join(HERE, "golden", "full_size_counts.json")))
KEYS = ("explored", "generated", "stored", "keys", "levels")


DL_ROWS = [r for r in ROWS if r["config"] == 2]
LT_ROWS = [r for r in ROWS if r["config"] == 3]


@pytest.mark.parametrize("row", LT_ROWS, ids=[f"config{r['config']}-seed{r['seed']}" for r in LT_ROWS])
def test_full_size_leadsto_query_matches_oracle(row):
    net, kind, p, q = config_instance(3, row["seed"])
    runs = []
    for _ in range(2):
        st = ReachStats()
        got = engine.leads_to_clocks(net, p, q, Backend.Cuda, st)
        assert got == row["holds"]
        runs.append({k: getattr(st, k) for k in KEYS})
    for k in KEYS:
        assert runs[0][k] == row[k], (k, runs[0][k], row[k])
    assert runs[1] == runs[0]


@pytest.mark.parametrize("row", DL_ROWS, ids=[f"config{r['config']}-seed{r['seed']}" for r in DL_ROWS])
def test_full_size_deadlock_query_matches_oracle(row):
    net = config_instance(row["config"], row["seed"])[0]
    runs = []
    for _ in range(2):
        st = ReachStats()
        got = engine.deadlock_reachable(net, Backend.Cuda, st)
        assert got == row["deadlock_reachable"]
        runs.append({k: getattr(st, k) for k in KEYS})
    for k in KEYS:
        assert runs[0][k] == row[k], (k, runs[0][k], row[k])
    assert runs[1] == runs[0]


SERVE_ROWS = [r for r in ROWS if r["config"] == 5]


@pytest.mark.skipif(not SERVE_ROWS, reason="no serving requests in the fixture")
def test_served_requests_match_oracle():
    """Requests of the serving workload's sequence (config-3 instances at full size) submitted
    together to the serving queue, so they overlap on the device: every verdict and count equals the
    oracle's for the same request run alone."""
    items = [config_instance(3, r["seed"]) for r in SERVE_ROWS]
    with engine.Server(budget_bytes=32 << 30, max_inflight=8) as srv:
        tickets = [srv.submit(*it) for it in items]
        srv.drain(timeout=600)
        got = [srv.poll(t) for t in tickets]
    for row, g in zip(SERVE_ROWS, got):
        assert g is not None, row["seed"]
        v, st = g
        assert st["status"] == 0, (row["seed"], st["status"])
        assert bool(v) == row["holds"], row["seed"]
        for k in KEYS:
            assert st[k] == row[k], (row["seed"], k, st[k], row[k])
