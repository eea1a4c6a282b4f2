"""The oracle's one-step functions of leads-to phase 2, used to replay counterexample traces: the
successor in the network restricted to !q lies inside the unrestricted successor by the same
transition and outside q, and equals it where q's discrete part fails; the stop set of a state is
classified as empty, its deadlocked valuations, or the whole zone."""
import numpy as np

from oracle import pyoracle
from ptctcl_gb300.generator import config_instance
from ptctcl_gb300.model import Pred


def _disc_ok(pred, locs, ints):
    for (pp, l) in pred.loc_req:
        if (locs[pp] != l) if l >= 0 else (locs[pp] == -l - 1):
            return False
    ops = {0: np.equal, 1: np.not_equal, 2: np.less, 3: np.less_equal, 4: np.greater, 5: np.greater_equal}
    return all(ops[op](ints[v], c) for (v, op, c) in pred.int_cond)


def test_restricted_successor_inside_unrestricted_and_outside_q():
    checked = restricted = 0
    for seed in range(6):
        net, kind, p, q0 = config_instance(3, seed)
        ok, l0, i0, z0 = pyoracle.initial_state(net)
        assert ok
        # q's clock atom at a location the first steps reach, so that the cut applies
        q = Pred([(0, int(l0[0]))], [], list(q0.clk_cond))
        frontier = [(l0, i0, z0)]
        for _ in range(3):
            nxt = []
            for (l, i, z) in frontier[:20]:
                for raw in range(40):
                    u = pyoracle.successor_raw(net, l, i, z, raw)
                    r = pyoracle.lt_successor_raw(net, q, l, i, z, raw)
                    if u is None:
                        assert r is None
                        continue
                    nxt.append(u)
                    if r is None:
                        continue
                    checked += 1
                    assert np.array_equal(r[0], u[0]) and np.array_equal(r[1], u[1])
                    assert (u[2] >= r[2]).all()                   # inside the unrestricted successor
                    if _disc_ok(q, r[0], r[1]):
                        restricted += 1
                        (a, b, v), = q.clk_cond
                        assert not pyoracle.Dbm(net.nclocks, r[2]).constrain(a, b, v)   # outside q
                    else:
                        assert np.array_equal(u[2], r[2])
                    assert pyoracle.lt_stop(net, q, r[0], r[1], r[2]) in (0, 1, 2)
            frontier = nxt
    assert checked > 50 and restricted > 0
