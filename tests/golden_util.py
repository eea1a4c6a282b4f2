"""Loading helpers for the committed golden fixtures (tests/golden)."""
import json
import os

from ptctcl_gb300.model import Network, query_from_json

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load_model(name: str) -> Network:
    with open(os.path.join(GOLDEN, "models", name + ".json")) as fh:
        return Network.from_json(json.load(fh))


def verdict_rows(kinds=(0, 1, 2)):
    with open(os.path.join(GOLDEN, "verdicts.json")) as fh:
        rows = json.load(fh)
    out = []
    for r in rows:
        kind, p, q = query_from_json(r["query"])
        if kind in kinds:
            out.append((r["model"], r["formula"], kind, p, q, r["result"]))
    return out


def toy_networks():
    """The two single-automaton models of tests/dbm_tests.cpp:77-124, as one-process networks."""
    from ptctcl_gb300.model import Process, Location, Edge, c_le, c_ge
    a = Location("A", [c_le(1, 10)])
    ta = Network(1, [Process("P", [a, Location("B"), Location("C")],
                             [Edge(0, 1, guard=[c_ge(1, 5)])], 0)], clock_names=["0", "x"])
    off, on = Location("Off"), Location("On", [c_le(1, 3)])
    t2 = Network(1, [Process("P", [off, on],
                             [Edge(0, 1, guard=[c_ge(1, 2)], resets=[1]),
                              Edge(1, 0, guard=[c_ge(1, 1)], resets=[1])], 0)], clock_names=["0", "x"])
    return ta, t2


def verdict_rows_dnf():
    """Rows whose formula has a top-level disjunction, lowered by the binding into several engine
    queries: (model, formula, combine, [(kind, p, q)], result) -- the recorded verdict is any (E<>,
    A<> as !E[]) or all (p --> q) of the terms' results (tests/golden/make_fixtures.py)."""
    with open(os.path.join(GOLDEN, "verdicts_dnf.json")) as fh:
        rows = json.load(fh)
    return [(r["model"], r["formula"], r["combine"], [query_from_json(t) for t in r["terms"]], r["result"])
            for r in rows]
