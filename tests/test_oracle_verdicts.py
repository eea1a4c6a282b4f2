"""Pin the oracle's whole-query results against the reference's recorded answers.

* tests/dbm_tests.cpp:77-124 -- reachability known answers on two one-automaton models;
* tests/uppaal-differential/round*.txt -- (model, formula) pairs on which HORA and UPPAAL verifyta
  agree, converted by tests/golden/make_fixtures.py.
"""
import os

import pytest

from oracle import pyoracle
from ptctcl_gb300.model import Pred, c_le, c_ge, c_gt
from golden_util import load_model, verdict_rows, verdict_rows_dnf, toy_networks


def test_dbm_tests_reachability():
    ta, t2 = toy_networks()
    R = lambda net, loc, cl=(): pyoracle.reachable_net(net, Pred([(0, loc)], [], list(cl)))[0]
    assert R(ta, 1)
    assert not R(ta, 2)
    assert not R(ta, 1, [c_le(1, 3)])
    assert R(ta, 1, [c_le(1, 8)])
    assert R(ta, 1, [c_ge(1, 5)])
    assert R(t2, 1)
    assert R(t2, 1, [c_le(1, 3)])
    assert not R(t2, 1, [c_gt(1, 3)])
    # the seq/omp agreement sweep of dbm_tests.cpp:116-123, checked against closed-form answers
    for L in range(3):
        for b in range(13):
            want_ta = {0: True, 1: b >= 5, 2: False}[L]
            assert R(ta, L, [c_le(1, b)]) == want_ta
            assert R(t2, L if L < 2 else 0, [c_le(1, b)]) is True


ROWS = verdict_rows(kinds=(0, 1))


@pytest.mark.parametrize("model,formula,kind,p,q,result", ROWS,
                         ids=[f"{r[0]}:{r[1]}" for r in ROWS])
def test_reference_verdicts(model, formula, kind, p, q, result):
    net = load_model(model)
    if kind == 0:
        got, st = pyoracle.reachable_net(net, p)
    else:
        got, st = pyoracle.deadlock_reachable(net)
    assert got == result, (formula, st)


# Rows whose exact zone graph is large (grc4 with T0.far on the right: 2e5-7e5 nodes) take 15-230 s
# in the single-threaded oracle; they run on the GPU tests and here only with HORA_SLOW_ORACLE=1.
SLOW = {("grc4", "x0 >= 0 --> T0.far"), ("grc4", "T0.in && x0 >= 0 --> T0.far"),
        ("grc4", "T0.in --> T0.far && x0 >= 0"), ("grc4", "T0.in --> T0.far")}
LT_ROWS = [r for r in verdict_rows(kinds=(2,))
           if (r[0], r[1]) not in SLOW or os.environ.get("HORA_SLOW_ORACLE") == "1"]


@pytest.mark.parametrize("model,formula,kind,p,q,result", LT_ROWS,
                         ids=[f"{r[0]}:{r[1]}" for r in LT_ROWS])
def test_reference_leadsto_verdicts(model, formula, kind, p, q, result):
    net = load_model(model)
    got, st = pyoracle.leads_to(net, p, q)
    assert got == result, (formula, st)


# E[] rows whose exact zone graph has 3e4-2e5 nodes take more than 5 s in the oracle; they run on the
# GPU tests and here only with HORA_SLOW_ORACLE=1.
EG_SLOW = {("grc4", "E[] x0 >= 0"), ("single4", "E[] x0 <= 3"), ("single4", "E[] x0 >= 0"),
           ("single4", "A<> x0 >= 3")}
EG_ROWS = [r for r in verdict_rows(kinds=(3,))
           if (r[0], r[1]) not in EG_SLOW or os.environ.get("HORA_SLOW_ORACLE") == "1"]


@pytest.mark.parametrize("model,formula,kind,p,q,result", EG_ROWS,
                         ids=[f"{r[0]}:{r[1]}" for r in EG_ROWS])
def test_reference_eg_verdicts(model, formula, kind, p, q, result):
    """E[] psi rows, and A<> phi rows run as E[] not phi (result = E[] not phi)."""
    net = load_model(model)
    got, st = pyoracle.exists_invariant(net, p)
    assert got == result, (formula, st)


# Disjunctive formulas, each term one oracle query: (p1 || p2) --> q holds iff every pi --> q holds;
# A<> (a1 || a2) with single-atom terms is !E[] (!a1 && !a2), one term. The grc4 rows run on the GPU
# tests and here only with HORA_SLOW_ORACLE=1.
DNF_ROWS = [r for r in verdict_rows_dnf() if r[0] != "grc4" or os.environ.get("HORA_SLOW_ORACLE") == "1"]


def oracle_term(net, kind, p, q):
    if kind == 0:
        return pyoracle.reachable_net(net, p)[0]
    if kind == 2:
        return pyoracle.leads_to(net, p, q)[0]
    return pyoracle.exists_invariant(net, p)[0]


@pytest.mark.parametrize("model,formula,combine,terms,result", DNF_ROWS,
                         ids=[f"{r[0]}:{r[1]}" for r in DNF_ROWS])
def test_reference_disjunctive_verdicts(model, formula, combine, terms, result):
    net = load_model(model)
    got = [oracle_term(net, k, p, q) for (k, p, q) in terms]
    assert (any(got) if combine == "any" else all(got)) == result, (formula, got)
