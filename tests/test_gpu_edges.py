"""Edge cases on the GPU, each against the oracle: networks without clocks, the largest DBM the
engine takes (16 clocks, 17 x 17), an initial state that violates its own invariant, an empty batch,
and a batch mixing every query kind with an instance the descriptor check rejects."""
import dataclasses

import numpy as np
import pytest

from oracle import pyoracle
from ptctcl_gb300 import capi, engine
from ptctcl_gb300 import generator as G
from ptctcl_gb300.engine import Backend, ReachStats
from ptctcl_gb300.model import (Network, Process, Location, Edge, Pred, c_le, clock_atom, Q_REACH, Q_DEADLOCK,
                                Q_LEADSTO, Q_EG)
from states import sample_states

pytestmark = pytest.mark.gpu

COUNTS = ("explored", "generated", "stored", "keys", "levels")


def _counts_equal(st, wst):
    for k in COUNTS:
        assert getattr(st, k) == wst[k], (k, getattr(st, k), wst[k])


def _net(nclocks, seed, nprocs=3, nlocs=4):
    rng = np.random.default_rng([99, nclocks, seed])
    g = dataclasses.replace(G.CONFIG_PARAMS[1], nprocs=nprocs, nlocs=nlocs, nclocks=nclocks)
    if nclocks == 0:   # integer guards and updates only
        g = dataclasses.replace(g, p_inv=0.0, guards_lo=0, guards_hi=0, p_reset=0.0, p_iguard=0.6, p_iupd=0.6)
    return G.random_network(rng, g), rng


@pytest.mark.parametrize("seed", range(4))
def test_no_clocks(seed):
    net, rng = _net(0, seed)
    target = Pred(G.two_locations(rng, net))
    st = ReachStats()
    assert engine.reachable_net(net, target, Backend.Cuda, st) == pyoracle.reachable_net(net, target)[0]
    st2 = ReachStats()
    got = engine.deadlock_reachable(net, Backend.Cuda, st2)
    want, wst = pyoracle.deadlock_reachable(net)
    assert got == want
    _counts_equal(st2, wst)


@pytest.mark.parametrize("seed", range(3))
def test_sixteen_clocks(seed):
    net, rng = _net(16, seed, nprocs=2, nlocs=4)
    smp = sample_states(net, nmax=60, depth=4)
    if smp is not None:
        locs, ints, zones, L, U = smp
        for emode in (0, 1):
            want = pyoracle.expand(net, locs, ints, zones, L, U, None, emode)
            got = engine.expand(net, locs, ints, zones, L, U, None, emode)
            for k in ("src", "ord", "locs", "ints", "zones"):
                np.testing.assert_array_equal(got[k], want[k], err_msg=k)
    target = Pred(G.two_locations(rng, net))
    st = ReachStats()
    got = engine.reachable_net(net, target, Backend.Cuda, st)
    want, wst = pyoracle.reachable_net(net, target)
    assert got == want
    _counts_equal(st, wst)


def test_initial_invariant_violated():
    # x < 0 at the initial location: there is no initial state at all
    net = Network(1, [Process("P", [Location("A", [clock_atom(1, "<", 0)]), Location("B")], [Edge(0, 1)], 0)],
                  clock_names=["0", "x"])
    st = ReachStats()
    assert engine.reachable_net(net, Pred([(0, 1)]), Backend.Cuda, st) is False
    assert pyoracle.reachable_net(net, Pred([(0, 1)]))[0] is False
    assert engine.deadlock_reachable(net, Backend.Cuda, ReachStats()) is False
    assert engine.exists_invariant_run(net, Pred([], [], [c_le(1, 5)]), Backend.Cuda) == \
        pyoracle.exists_invariant(net, Pred([], [], [c_le(1, 5)]))[0]


def test_empty_batch():
    verdicts, stats = engine.batch_run([])
    assert verdicts == [] and stats == []


def test_batch_mixes_every_kind_and_a_rejected_instance():
    net, rng = _net(3, 7)
    items = [(net, Q_REACH, Pred(G.two_locations(rng, net)), Pred()),
             (net, Q_DEADLOCK, Pred(), Pred()),
             (net, Q_LEADSTO, Pred([(0, 1)]), Pred([(1, 2)])),
             (net, Q_EG, Pred([], [], [c_le(1, 10)]), Pred()),
             (net, Q_REACH, Pred([(0, 99)]), Pred())]   # location out of range
    verdicts, stats = engine.batch_run(items)
    assert stats[4]["status"] == capi.E_INVALID and verdicts[4] == -1
    assert verdicts[0] == int(pyoracle.reachable_net(net, items[0][2])[0])
    assert verdicts[1] == int(pyoracle.deadlock_reachable(net)[0])
    assert verdicts[2] == int(pyoracle.leads_to(net, items[2][2], items[2][3])[0])
    assert verdicts[3] == int(pyoracle.exists_invariant(net, items[3][2])[0])
    assert all(s["status"] == capi.OK for s in stats[:4])
