"""E[] psi witnesses emitted by the GPU, replayed through the oracle's successor function of the
psi-restricted graph: step 0 is the restricted initial state, every later step is the successor of
the one before with the recorded emission ordinal, and a closing edge leads back into the path. A
psi that fails has no witness."""
import numpy as np
import pytest

from oracle import pyoracle
from ptctcl_gb300 import engine
from ptctcl_gb300.engine import Backend
from golden_util import load_model, verdict_rows

pytestmark = pytest.mark.gpu

SLOW = {("grc4", "E[] x0 >= 0"), ("single4", "E[] x0 <= 3"), ("single4", "E[] x0 >= 0"), ("single4", "A<> x0 >= 3")}
ROWS = [r for r in verdict_rows(kinds=(3,)) if (r[0], r[1]) not in SLOW]


def _same(a, b):
    return all(np.array_equal(np.asarray(x), np.asarray(y)) for x, y in zip(a, b))


@pytest.mark.parametrize("model,formula,kind,p,q,result", ROWS, ids=[f"{r[0]}:{r[1]}" for r in ROWS])
def test_eg_witness_replays(model, formula, kind, p, q, result):
    net = load_model(model)
    holds, tr = engine.exists_invariant_trace(net, p, Backend.Cuda)
    assert holds == result
    if not holds:
        assert tr is None
        return
    n = len(tr["ords"])
    assert n >= 1 and tr["ords"][0] == -1
    init = pyoracle.eg_initial(net, p)
    assert init is not None
    assert _same(init, (tr["locs"][0], tr["ints"][0], tr["zones"][0]))
    for i in range(1, n):
        sl, si, sz = pyoracle.eg_successors(net, p, tr["locs"][i - 1], tr["ints"][i - 1], tr["zones"][i - 1])
        k = tr["ords"][i]
        assert 0 <= k < len(sz), (i, k, len(sz))
        assert _same((sl[k], si[k], sz[k]), (tr["locs"][i], tr["ints"][i], tr["zones"][i])), i
    if tr["loop_to"] >= 0:
        sl, si, sz = pyoracle.eg_successors(net, p, tr["locs"][n - 1], tr["ints"][n - 1], tr["zones"][n - 1])
        k, j = tr["loop_ord"], tr["loop_to"]
        assert 0 <= k < len(sz) and 0 <= j < n
        assert _same((sl[k], si[k], sz[k]), (tr["locs"][j], tr["ints"][j], tr["zones"][j]))


# ---- counterexamples of the forward routes: reach, deadlock, the leads-to early witness ----
from ptctcl_gb300.generator import config_instance  # noqa: E402
from ptctcl_gb300.model import Q_REACH, Q_DEADLOCK, Q_LEADSTO  # noqa: E402
from test_gpu_parity import small_config3  # noqa: E402


def _qmask(net, *preds):
    """The clocks the query reads (kept by the active-clock reduction), as the engine folds them in."""
    m = np.zeros(net.dim, np.uint8)
    for pr in preds:
        for (i, j, _) in pr.clk_cond:
            m[i] = m[j] = 1
    m[0] = 0
    return m


def _disc_ok(pred, locs, ints):
    for (pp, l) in pred.loc_req:
        if (locs[pp] != l) if l >= 0 else (locs[pp] == -l - 1):
            return False
    ops = {0: np.equal, 1: np.not_equal, 2: np.less, 3: np.less_equal, 4: np.greater, 5: np.greater_equal}
    return all(ops[op](ints[v], c) for (v, op, c) in pred.int_cond)


CASES = ([("c1", 1, s) for s in range(12)] + [("c2", 2, s) for s in (0, 3, 10, 23)] +
         [("c4", 4, s) for s in (0, 1, 2, 3, 4, 5, 8, 9, 12, 13, 14, 18, 19, 22, 23, 25, 26, 75)] +
         [("c3", 3, s) for s in (0, 1, 13, 19, 20, 33)] +
         # violations decided by the backward sweep (no early witness)
         [("c3", 3, s) for s in (14, 17, 23, 25, 37, 39)])


def _check_sweep_trace(net, p, q, qm, tr):
    """A leads-to counterexample found by the backward sweep: the passed-store path from the initial
    state to a p-state (as for the forward routes), the root (ords -2) inside that state cut to p and
    !q, then steps of the network restricted to !q -- each the oracle's restricted successor of the
    step before by the recorded transition, inside the step's zone, outside q -- ending at a state
    whose stop set is not empty or closing a cycle by a restricted successor inside the step it
    returns to."""
    ords = tr["ords"]
    n = len(ords)
    r = ords.index(-2)
    assert r >= 1 and ords.count(-2) == 1 and ords[0] == -1
    ok, l0, i0, z0 = pyoracle.initial_state(net, qm)
    assert ok and np.array_equal(l0, tr["locs"][0]) and np.array_equal(i0, tr["ints"][0])
    assert (tr["zones"][0] >= z0).all()
    for i in range(1, r):
        succ = pyoracle.successor_raw(net, tr["locs"][i - 1], tr["ints"][i - 1], tr["zones"][i - 1], ords[i], qm)
        assert succ is not None, i
        sl, si, sz = succ
        assert np.array_equal(sl, tr["locs"][i]) and np.array_equal(si, tr["ints"][i]), i
        assert (tr["zones"][i] >= sz).all(), i
    # the root: the same discrete state, a p-state outside q's discrete part or cut by q's clock atom
    assert np.array_equal(tr["locs"][r], tr["locs"][r - 1]) and np.array_equal(tr["ints"][r], tr["ints"][r - 1])
    assert _disc_ok(p, tr["locs"][r], tr["ints"][r])
    cut = pyoracle.Dbm(net.nclocks, tr["zones"][r - 1])
    assert all(cut.constrain(i, j, v) for (i, j, v) in p.clk_cond)
    in_q = _disc_ok(q, tr["locs"][r], tr["ints"][r])
    assert not (in_q and not q.clk_cond)
    for i in range(r, n):
        if _disc_ok(q, tr["locs"][i], tr["ints"][i]):
            # every valuation of a !q-graph zone lies outside q's clock atom
            (a, b, v), = q.clk_cond
            d = pyoracle.Dbm(net.nclocks, tr["zones"][i])
            assert not d.constrain(a, b, v), i
    for i in range(r + 1, n):
        succ = pyoracle.lt_successor_raw(net, q, tr["locs"][i - 1], tr["ints"][i - 1], tr["zones"][i - 1], ords[i], qm)
        assert succ is not None, i
        sl, si, sz = succ
        assert np.array_equal(sl, tr["locs"][i]) and np.array_equal(si, tr["ints"][i]), i
        assert (tr["zones"][i] >= sz).all(), i
    if tr["loop_to"] >= 0:
        j = tr["loop_to"]
        assert r <= j < n
        succ = pyoracle.lt_successor_raw(net, q, tr["locs"][n - 1], tr["ints"][n - 1], tr["zones"][n - 1],
                                         tr["loop_ord"], qm)
        assert succ is not None
        sl, si, sz = succ
        assert np.array_equal(sl, tr["locs"][j]) and np.array_equal(si, tr["ints"][j])
        assert (tr["zones"][j] >= sz).all()
    else:
        assert pyoracle.lt_stop(net, q, tr["locs"][n - 1], tr["ints"][n - 1], tr["zones"][n - 1], qm) > 0


@pytest.mark.parametrize("name,cfg,seed", CASES, ids=[f"{n}-{s}" for n, _, s in CASES])
def test_counterexample_replays(name, cfg, seed):
    """When the goal is reached, the trace is a path of the passed store: step 0 is the initial state,
    the oracle's exact successor of step i-1 by transition ords[i] exists, has step i's discrete state
    and lies inside step i's stored zone, and the last step is a goal state (a target state, a state
    holding a deadlocked valuation, or a p-state for the leads-to witness)."""
    net, kind, p, q = small_config3(seed) if cfg == 3 else config_instance(cfg, seed)
    with engine.QueryHandle(net, kind, p, q) as h:
        verdict = h.run()
        tr = h.trace()
    goal = verdict if kind in (Q_REACH, Q_DEADLOCK) else not verdict
    if not goal:
        assert tr is None
        return
    assert tr is not None
    qm = _qmask(net, p) if kind == Q_REACH else _qmask(net, p, q) if kind == Q_LEADSTO else _qmask(net)
    if kind == Q_LEADSTO and -2 in tr["ords"]:
        _check_sweep_trace(net, p, q, qm, tr)
        return
    n = len(tr["ords"])
    assert tr["ords"][0] == -1 and tr["loop_to"] == -1
    ok, l0, i0, z0 = pyoracle.initial_state(net, qm)
    assert ok
    assert np.array_equal(l0, tr["locs"][0]) and np.array_equal(i0, tr["ints"][0])
    assert (tr["zones"][0] >= z0).all()
    for i in range(1, n):
        succ = pyoracle.successor_raw(net, tr["locs"][i - 1], tr["ints"][i - 1], tr["zones"][i - 1], tr["ords"][i], qm)
        assert succ is not None, i
        sl, si, sz = succ
        assert np.array_equal(sl, tr["locs"][i]) and np.array_equal(si, tr["ints"][i]), i
        assert (tr["zones"][i] >= sz).all(), i          # the stored zone contains the exact successor
    fl, fi, fz = tr["locs"][-1], tr["ints"][-1], tr["zones"][-1]
    if kind == Q_REACH:
        assert _disc_ok(p, fl, fi)
        d = pyoracle.Dbm(net.nclocks, fz)
        assert all(d.constrain(i, j, r) for (i, j, r) in p.clk_cond)
    elif kind == Q_DEADLOCK:
        assert pyoracle.has_deadlock(net, fl[None, :], fi[None, :], fz[None, :])[0]
    else:
        assert _disc_ok(p, fl, fi) and not (q.clk_cond == [] and _disc_ok(q, fl, fi))
