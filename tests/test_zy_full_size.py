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
