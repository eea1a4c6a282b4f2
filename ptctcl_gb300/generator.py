"""Seeded synthetic networks and queries with the shapes of the benchmark configurations.

The reference ships no generator for networks (its tests/difftest_ta.py:21-60 draws single
automata only), so this one follows the published configuration text literally:

* ``config1`` -- 3 automata x 6 locations, 4 clocks (5x5 DBM), 2 ints in [0,3]; every location has
  2-4 outgoing edges, each with 1-2 clock guards ``x ~ c`` (~ uniform over <,<=,>=,>; c in
  [0,20]), every clock reset with p=0.3, a sync on one of 2 binary channels with p=0.3 (sender or
  receiver uniformly); 50% of locations carry an invariant ``x <= c``, c in [5,20]. Query
  ``E<>`` of two random locations.
* ``config2`` -- the same with 8 automata x 10 locations, 8 clocks (9x9 DBM), 4 binary channels
  and 1 broadcast channel, 10% committed and 10% urgent locations, c in [0,50]. Query
  ``A[] not deadlock``.
* ``config3`` -- 6 automata x 8 locations, 6 clocks (7x7 DBM), c in [0,30]. Query ``p --> q``, p and
  q each a conjunction of two locations plus one clock atom (never ``==``).
* ``config4`` -- clocks U[2,16], automata U[2,10], locations U[4,12], c in [0,40]; query mix
  60% ``E<>`` / 30% deadlock / 10% leads-to.

Choices the text leaves open, fixed here: integer guards ``v OP k`` on an edge with p=0.2 and
integer updates ``v := k`` with p=0.2; edge targets uniform over the automaton's locations;
guard clocks uniform over all clocks; initial location 0; integers start at 0.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .model import (Network, Process, Location, Edge, IntVar, Pred, clock_atom, c_le,
                    CHAN_BROADCAST, Q_REACH, Q_DEADLOCK, Q_LEADSTO)

OPS = ("<", "<=", ">=", ">")
IOPS = (0, 1, 2, 3, 4, 5)


@dataclass
class GenParams:
    nprocs: int
    nlocs: int
    nclocks: int
    nints: int = 2
    int_hi: int = 3
    n_binary: int = 2
    n_broadcast: int = 0
    cmax: int = 20
    inv_lo: int = 5
    inv_hi: int = 20
    p_inv: float = 0.5
    p_committed: float = 0.0
    p_urgent: float = 0.0
    p_reset: float = 0.3
    p_sync: float = 0.3
    p_iguard: float = 0.2
    p_iupd: float = 0.2
    edges_lo: int = 2
    edges_hi: int = 4
    guards_lo: int = 1
    guards_hi: int = 2


def random_network(rng: np.random.Generator, g: GenParams) -> Network:
    nch = g.n_binary + g.n_broadcast
    chans = [(f"c{k}", 0) for k in range(g.n_binary)] + [(f"b{k}", CHAN_BROADCAST) for k in range(g.n_broadcast)]
    ints = [IntVar(f"v{k}", 0, g.int_hi, 0) for k in range(g.nints)]
    procs = []
    for p in range(g.nprocs):
        locs = []
        for l in range(g.nlocs):
            inv = []
            if rng.random() < g.p_inv:
                inv.append(c_le(int(rng.integers(1, g.nclocks + 1)), int(rng.integers(g.inv_lo, g.inv_hi + 1))))
            r = rng.random()
            committed = r < g.p_committed
            urgent = (not committed) and r < g.p_committed + g.p_urgent
            locs.append(Location(f"L{l}", inv, urgent, committed))
        edges = []
        for l in range(g.nlocs):
            for _ in range(int(rng.integers(g.edges_lo, g.edges_hi + 1))):
                e = Edge(l, int(rng.integers(0, g.nlocs)))
                for _k in range(int(rng.integers(g.guards_lo, g.guards_hi + 1))):
                    e.guard.append(clock_atom(int(rng.integers(1, g.nclocks + 1)), OPS[int(rng.integers(0, 4))],
                                              int(rng.integers(0, g.cmax + 1))))
                if g.nints and rng.random() < g.p_iguard:
                    e.iguard.append((int(rng.integers(0, g.nints)), IOPS[int(rng.integers(0, 6))],
                                     int(rng.integers(0, g.int_hi + 1))))
                e.resets = [c for c in range(1, g.nclocks + 1) if rng.random() < g.p_reset]
                if g.nints and rng.random() < g.p_iupd:
                    e.iupd.append((int(rng.integers(0, g.nints)), int(rng.integers(0, g.int_hi + 1))))
                if nch and rng.random() < g.p_sync:
                    e.chan = int(rng.integers(0, nch))
                    e.dir = 1 if rng.random() < 0.5 else -1
                edges.append(e)
        procs.append(Process(f"P{p}", locs, edges, 0))
    return Network(g.nclocks, procs, ints, chans, ["0"] + [f"x{c}" for c in range(1, g.nclocks + 1)])


def two_locations(rng, net: Network):
    ps = rng.choice(len(net.procs), size=2, replace=False)
    return [(int(p), int(rng.integers(0, len(net.procs[p].locations)))) for p in sorted(ps)]


def clock_term(rng, net: Network, cmax: int):
    return clock_atom(int(rng.integers(1, net.nclocks + 1)), OPS[int(rng.integers(0, 4))],
                      int(rng.integers(0, cmax + 1)))


CONFIG_PARAMS = {
    1: GenParams(nprocs=3, nlocs=6, nclocks=4, n_binary=2, cmax=20),
    2: GenParams(nprocs=8, nlocs=10, nclocks=8, n_binary=4, n_broadcast=1, cmax=50,
                 p_committed=0.1, p_urgent=0.1),
    3: GenParams(nprocs=6, nlocs=8, nclocks=6, n_binary=2, cmax=30),
}


def config_instance(config: int, seed: int):
    """-> (Network, kind, p, q) for one seeded instance of configuration 1, 2, 3 or 4."""
    rng = np.random.default_rng([config, seed])
    if config in (1, 2, 3):
        net = random_network(rng, CONFIG_PARAMS[config])
        if config == 1:
            return net, Q_REACH, Pred(two_locations(rng, net)), Pred()
        if config == 2:
            return net, Q_DEADLOCK, Pred(), Pred()
        p = Pred(two_locations(rng, net), [], [clock_term(rng, net, 30)])
        q = Pred(two_locations(rng, net), [], [clock_term(rng, net, 30)])
        return net, Q_LEADSTO, p, q
    if config == 4:
        g = GenParams(nprocs=int(rng.integers(2, 11)), nlocs=int(rng.integers(4, 13)),
                      nclocks=int(rng.integers(2, 17)), n_binary=2, cmax=40)
        net = random_network(rng, g)
        r = rng.random()
        if r < 0.6:
            return net, Q_REACH, Pred(two_locations(rng, net)), Pred()
        if r < 0.9:
            return net, Q_DEADLOCK, Pred(), Pred()
        p = Pred(two_locations(rng, net), [], [clock_term(rng, net, 40)])
        q = Pred(two_locations(rng, net), [], [clock_term(rng, net, 40)])
        return net, Q_LEADSTO, p, q
    raise ValueError(config)


def to_uppaal_xml(net: Network) -> str:
    """The network as flat UPPAAL XML, the form the reference's load_network reads."""
    def cname(c):
        return net.clock_names[c] if net.clock_names else f"x{c}"

    def cons(cs):
        out = []
        for i, j, raw in cs:
            v, strict = raw >> 1, (raw & 1) == 0
            if j == 0:
                out.append(f"{cname(i)} {'&lt;' if strict else '&lt;='} {v}")
            elif i == 0:
                out.append(f"{cname(j)} {'&gt;' if strict else '&gt;='} {-v}")
            else:
                out.append(f"{cname(i)} - {cname(j)} {'&lt;' if strict else '&lt;='} {v}")
        return out
    iop = ["==", "!=", "&lt;", "&lt;=", "&gt;", "&gt;="]
    lines = ['<?xml version="1.0" encoding="utf-8"?>', "<nta>"]
    decl = []
    if net.nclocks:
        decl.append("clock " + ",".join(cname(c) for c in range(1, net.nclocks + 1)) + ";")
    for v in net.ints:
        decl.append(f"int[{v.lo},{v.hi}] {v.name} = {v.init};")
    for name, fl in net.chans:
        decl.append(("urgent " if fl & 2 else "") + ("broadcast " if fl & 1 else "") + f"chan {name};")
    lines.append("<declaration>" + " ".join(decl) + "</declaration>")
    for p in net.procs:
        lines.append(f"<template><name>{p.name}</name>")
        for k, l in enumerate(p.locations):
            inv = cons(l.invariant)
            lab = f'<label kind="invariant">{" &amp;&amp; ".join(inv)}</label>' if inv else ""
            flag = "<urgent/>" if l.urgent else ("<committed/>" if l.committed else "")
            lines.append(f'<location id="{p.name}_{k}"><name>{l.name}</name>{lab}{flag}</location>')
        lines.append(f'<init ref="{p.name}_{p.initial}"/>')
        for e in p.edges:
            g = cons(e.guard) + [f"{net.ints[v].name} {iop[op]} {k}" for v, op, k in e.iguard]
            a = [f"{cname(r)} = 0" for r in e.resets] + [f"{net.ints[v].name} = {k}" for v, k in e.iupd]
            s = f'<transition><source ref="{p.name}_{e.src}"/><target ref="{p.name}_{e.tgt}"/>'
            if g:
                s += f'<label kind="guard">{" &amp;&amp; ".join(g)}</label>'
            if e.chan >= 0:
                s += f'<label kind="synchronisation">{net.chans[e.chan][0]}{"!" if e.dir > 0 else "?"}</label>'
            if a:
                s += f'<label kind="assignment">{", ".join(a)}</label>'
            lines.append(s + "</transition>")
        lines.append("</template>")
    lines.append("<system>system " + ", ".join(p.name for p in net.procs) + ";</system></nta>")
    return "\n".join(lines)
