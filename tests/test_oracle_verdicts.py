"""Pin the oracle's whole-query results against the reference's recorded answers.

* tests/dbm_tests.cpp:77-124 -- reachability known answers on two one-automaton models;
* tests/uppaal-differential/round*.txt -- (model, formula) pairs on which HORA and UPPAAL verifyta
  agree, converted by tests/golden/make_fixtures.py.
"""
import pytest

from oracle import pyoracle
from ptctcl_gb300.model import Pred, c_le, c_ge, c_gt
from golden_util import load_model, verdict_rows, toy_networks


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
