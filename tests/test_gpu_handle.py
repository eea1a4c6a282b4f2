"""The handle form (hora_gb_open / run / trace / close): a query opened once runs with the verdict
and counts of the matching single-query entry point, again on every run, from descriptors the
caller has already dropped; an E[] handle keeps the same witness as hora_gb_exists_invariant_trace."""
import gc

import numpy as np
import pytest

from ptctcl_gb300 import engine
from ptctcl_gb300.engine import Backend, ReachStats, QueryHandle
from golden_util import load_model, verdict_rows

pytestmark = pytest.mark.gpu

SLOW = {("grc4", "E[] x0 >= 0"), ("single4", "E[] x0 <= 3"), ("single4", "E[] x0 >= 0"),
        ("single4", "A<> x0 >= 3"), ("grc4", "x0 >= 0 --> T0.far"), ("grc4", "T0.in && x0 >= 0 --> T0.far"),
        ("grc4", "T0.in --> T0.far && x0 >= 0"), ("grc4", "T0.in --> T0.far")}
ROWS = []
for kind in (0, 1, 2, 3):
    ROWS += [r for r in verdict_rows(kinds=(kind,)) if (r[0], r[1]) not in SLOW][:6]
COUNTS = ("explored", "generated", "stored", "levels")


def _direct(net, kind, p, q, st):
    if kind == 0:
        return engine.reachable_net(net, p, Backend.Cuda, st)
    if kind == 1:
        return engine.deadlock_reachable(net, Backend.Cuda, st)
    if kind == 2:
        return engine.leads_to_clocks(net, p, q, Backend.Cuda, st)
    return engine.exists_invariant_run(net, p, Backend.Cuda, st)


@pytest.mark.parametrize("model,formula,kind,p,q,result", ROWS, ids=[f"{r[0]}:{r[1]}" for r in ROWS])
def test_handle_matches_single_query_entry_points(model, formula, kind, p, q, result):
    net = load_model(model)
    want_st = ReachStats()
    want = _direct(net, kind, p, q, want_st)
    h = QueryHandle(net, kind, p, q)
    gc.collect()   # the descriptors built for hora_gb_open are gone; the handle holds its own copy
    for _ in range(2):
        st = ReachStats()
        assert h.run(st) == want
        for c in COUNTS:
            assert getattr(st, c) == getattr(want_st, c), c
    if kind == 3:
        holds, tr = engine.exists_invariant_trace(net, p, Backend.Cuda)
        got = h.trace()
        assert holds == want
        if tr is None:
            assert got is None
        else:
            assert got["ords"] == tr["ords"] and got["loop_to"] == tr["loop_to"] and got["loop_ord"] == tr["loop_ord"]
            for f in ("locs", "ints", "zones"):
                assert np.array_equal(got[f], tr[f]), f
    h.close()
