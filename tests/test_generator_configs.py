"""The seeded generator produces the benchmark configurations' shapes: automata, locations,
clocks, channels, integer ranges, guard and invariant constants, committed / urgent shares and the
query mix, and the same instance for the same seed."""
import numpy as np
import pytest

from ptctcl_gb300.generator import config_instance
from ptctcl_gb300.model import CHAN_BROADCAST, Q_REACH, Q_DEADLOCK, Q_LEADSTO

SHAPES = {1: (3, 6, 4, 2, 0, 20), 2: (8, 10, 8, 4, 1, 50), 3: (6, 8, 6, 2, 0, 30)}


def _bound(atom):
    return abs(atom[2] >> 1)


def _check_network(net, nprocs, nlocs, nclocks, nbin, nbc, cmax):
    assert len(net.procs) == nprocs and net.nclocks == nclocks and net.dim == nclocks + 1
    assert [f for _, f in net.chans].count(CHAN_BROADCAST) == nbc and len(net.chans) == nbin + nbc
    assert len(net.ints) == 2 and all(v.lo == 0 and v.hi == 3 and v.init == 0 for v in net.ints)
    for pr in net.procs:
        assert len(pr.locations) == nlocs and pr.initial == 0
        out = np.bincount([e.src for e in pr.edges], minlength=nlocs)
        assert out.min() >= 2 and out.max() <= 4
        for loc in pr.locations:
            assert len(loc.invariant) <= 1
            for a in loc.invariant:
                assert a[1] == 0 and 5 <= (a[2] >> 1) <= 20 and (a[2] & 1) == 1   # x <= c, c in [5,20]
            assert not (loc.urgent and loc.committed)
        for e in pr.edges:
            assert 1 <= len(e.guard) <= 2 and all(_bound(a) <= cmax for a in e.guard)
            assert all(1 <= c <= nclocks for c in e.resets)
            assert e.chan == -1 or (0 <= e.chan < nbin + nbc and e.dir in (1, -1))


@pytest.mark.parametrize("config", [1, 2, 3])
def test_fixed_configurations(config):
    nprocs, nlocs, nclocks, nbin, nbc, cmax = SHAPES[config]
    urgent = committed = total = 0
    for seed in range(20):
        net, kind, p, q = config_instance(config, seed)
        _check_network(net, nprocs, nlocs, nclocks, nbin, nbc, cmax)
        for pr in net.procs:
            urgent += sum(l.urgent for l in pr.locations)
            committed += sum(l.committed for l in pr.locations)
            total += len(pr.locations)
        if config == 1:
            assert kind == Q_REACH and len(p.loc_req) == 2 and p.loc_req[0][0] != p.loc_req[1][0]
        elif config == 2:
            assert kind == Q_DEADLOCK
        else:
            assert kind == Q_LEADSTO
            for side in (p, q):
                assert len(side.loc_req) == 2 and len(side.clk_cond) == 1 and _bound(side.clk_cond[0]) <= 30
    if config == 2:
        assert 0.07 <= committed / total <= 0.13 and 0.07 <= urgent / total <= 0.13
    else:
        assert committed == 0 and urgent == 0


def test_config4_ranges_and_query_mix():
    kinds = []
    for seed in range(1500):
        net, kind, p, q = config_instance(4, seed)
        assert 2 <= len(net.procs) <= 10 and 2 <= net.nclocks <= 16
        nl = len(net.procs[0].locations)
        assert 4 <= nl <= 12 and all(len(pr.locations) == nl for pr in net.procs)
        for pr in net.procs:
            for e in pr.edges:
                assert all(_bound(a) <= 40 for a in e.guard)
        kinds.append(kind)
    kinds = np.array(kinds)
    assert abs(np.mean(kinds == Q_REACH) - 0.6) < 0.04
    assert abs(np.mean(kinds == Q_DEADLOCK) - 0.3) < 0.04
    assert abs(np.mean(kinds == Q_LEADSTO) - 0.1) < 0.03


@pytest.mark.parametrize("config", [1, 2, 3, 4])
def test_same_seed_same_instance(config):
    a, b = config_instance(config, 5), config_instance(config, 5)
    assert a[1] == b[1] and a[0] == b[0] and a[2] == b[2] and a[3] == b[3]
    c = config_instance(config, 6)
    assert c[0] != a[0]
