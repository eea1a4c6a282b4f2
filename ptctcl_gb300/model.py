"""Network-of-timed-automata model and its flattened C-ABI descriptor.

The classes mirror the reference's model IR (include/hora/network.hpp:19-140,
include/hora/automaton.hpp:15-30): a network has shared clocks (index 0 is the constant-zero
reference clock), bounded integer variables, binary/broadcast/urgent channels and one process
per automaton. Only the fast-path forms of guards and updates exist -- ``var OP const`` and
``var := const`` -- which is what ``NEdge::int_guard``/``int_updates`` hold; general expressions
(``NEdge::gen_guard``) are not representable here.

Clock constraints are ``(i, j, raw)`` triples meaning ``x_i - x_j <| bound`` with
``raw = (bound << 1) | weak`` (HDBM's encoding, src/metal/netengine_metal.mm:91-100).
"""
from __future__ import annotations

import ctypes
import json
from dataclasses import dataclass, field
from typing import List, Sequence, Tuple

import numpy as np

INF = 1 << 30
ZERO_LE = 1
ALU_NEG_INF = -(1 << 29)

IOP = {"==": 0, "!=": 1, "<": 2, "<=": 3, ">": 4, ">=": 5}
CHAN_BROADCAST = 1
CHAN_URGENT = 2
LOC_URGENT = 1
LOC_COMMITTED = 2


def le(v: int) -> int:
    return (v << 1) | 1


def lt(v: int) -> int:
    return v << 1


def raw_bound(r: int) -> int:
    return r >> 1


def raw_strict(r: int) -> bool:
    return (r & 1) == 0


def c_le(x: int, v: int) -> Tuple[int, int, int]:
    """x <= v"""
    return (x, 0, le(v))


def c_lt(x: int, v: int) -> Tuple[int, int, int]:
    """x < v"""
    return (x, 0, lt(v))


def c_ge(x: int, v: int) -> Tuple[int, int, int]:
    """x >= v, i.e. 0 - x <= -v"""
    return (0, x, le(-v))


def c_gt(x: int, v: int) -> Tuple[int, int, int]:
    """x > v, i.e. 0 - x < -v"""
    return (0, x, lt(-v))


def clock_atom(x: int, op: str, v: int) -> Tuple[int, int, int]:
    return {"<=": c_le, "<": c_lt, ">=": c_ge, ">": c_gt}[op](x, v)


@dataclass
class Location:
    name: str
    invariant: List[Tuple[int, int, int]] = field(default_factory=list)
    urgent: bool = False
    committed: bool = False


@dataclass
class Edge:
    src: int
    tgt: int
    guard: List[Tuple[int, int, int]] = field(default_factory=list)
    iguard: List[Tuple[int, int, int]] = field(default_factory=list)   # (var, op, val)
    resets: List[int] = field(default_factory=list)
    iupd: List[Tuple[int, int]] = field(default_factory=list)          # (var, val)
    chan: int = -1
    dir: int = 0                                                        # +1 a!, -1 a?


@dataclass
class Process:
    name: str
    locations: List[Location]
    edges: List[Edge]
    initial: int = 0


@dataclass
class IntVar:
    name: str
    lo: int
    hi: int
    init: int = 0


@dataclass
class Network:
    nclocks: int
    procs: List[Process]
    ints: List[IntVar] = field(default_factory=list)
    chans: List[Tuple[str, int]] = field(default_factory=list)        # (name, HORA_CHAN_* flags)
    clock_names: List[str] = field(default_factory=list)

    @property
    def dim(self) -> int:
        return self.nclocks + 1

    def loc_index(self, proc: str, loc: str) -> Tuple[int, int]:
        for p, pr in enumerate(self.procs):
            if pr.name == proc:
                for l, lo in enumerate(pr.locations):
                    if lo.name == loc:
                        return p, l
        raise KeyError(f"{proc}.{loc}")

    def key_bits(self) -> int:
        def fb(n):
            b = 0
            while (1 << b) < n:
                b += 1
            return b
        return sum(fb(len(p.locations)) for p in self.procs) + sum(fb(v.hi - v.lo + 1) for v in self.ints)

    # ---- (de)serialisation, used for fixtures -------------------------------------------------
    def to_json(self) -> dict:
        return {
            "nclocks": self.nclocks,
            "clock_names": self.clock_names,
            "ints": [[v.name, v.lo, v.hi, v.init] for v in self.ints],
            "chans": [[c, f] for c, f in self.chans],
            "procs": [{
                "name": p.name, "initial": p.initial,
                "locations": [[l.name, [list(c) for c in l.invariant], int(l.urgent), int(l.committed)]
                              for l in p.locations],
                "edges": [[e.src, e.tgt, [list(c) for c in e.guard], [list(a) for a in e.iguard],
                           list(e.resets), [list(u) for u in e.iupd], e.chan, e.dir] for e in p.edges],
            } for p in self.procs],
        }

    @staticmethod
    def from_json(d: dict) -> "Network":
        procs = []
        for p in d["procs"]:
            locs = [Location(n, [tuple(c) for c in inv], bool(u), bool(cm)) for n, inv, u, cm in p["locations"]]
            edges = [Edge(s, t, [tuple(c) for c in g], [tuple(a) for a in ig], list(r), [tuple(u) for u in iu], ch, dr)
                     for s, t, g, ig, r, iu, ch, dr in p["edges"]]
            procs.append(Process(p["name"], locs, edges, p["initial"]))
        return Network(d["nclocks"], procs, [IntVar(*v) for v in d["ints"]],
                       [tuple(c) for c in d["chans"]], list(d.get("clock_names", [])))

    def dumps(self) -> str:
        return json.dumps(self.to_json(), separators=(",", ":"))


@dataclass
class Pred:
    """A conjunction of location, integer and clock atoms (NetTarget / DiscPred conjunction)."""
    loc_req: List[Tuple[int, int]] = field(default_factory=list)
    int_cond: List[Tuple[int, int, int]] = field(default_factory=list)
    clk_cond: List[Tuple[int, int, int]] = field(default_factory=list)
    never: bool = False

    def to_json(self):
        return {"loc": [list(x) for x in self.loc_req], "int": [list(x) for x in self.int_cond],
                "clk": [list(x) for x in self.clk_cond], "never": int(self.never)}

    @staticmethod
    def from_json(d):
        return Pred([tuple(x) for x in d["loc"]], [tuple(x) for x in d["int"]],
                    [tuple(x) for x in d["clk"]], bool(d.get("never", 0)))


# ---------------------------------------------------------------------------------------------
# C-ABI structures (include/hora_gb300.h)
# ---------------------------------------------------------------------------------------------
P32 = ctypes.POINTER(ctypes.c_int32)


class NetDesc(ctypes.Structure):
    _fields_ = [
        ("nclocks", ctypes.c_int32), ("nprocs", ctypes.c_int32), ("nints", ctypes.c_int32),
        ("nchans", ctypes.c_int32), ("chan_flags", P32), ("int_lo", P32), ("int_hi", P32),
        ("int_init", P32), ("proc_nlocs", P32), ("proc_init", P32), ("loc_flags", P32),
        ("loc_inv_off", P32), ("nedges", ctypes.c_int32), ("edge_proc", P32), ("edge_src", P32),
        ("edge_tgt", P32), ("edge_chan", P32), ("edge_dir", P32), ("edge_guard_off", P32),
        ("edge_iguard_off", P32), ("edge_reset_off", P32), ("edge_iupd_off", P32), ("cons", P32),
        ("iatoms", P32), ("resets", P32), ("iupds", P32),
    ]


class PredDesc(ctypes.Structure):
    _fields_ = [("nloc", ctypes.c_int32), ("loc_req", P32), ("nint", ctypes.c_int32),
                ("int_cond", P32), ("nclk", ctypes.c_int32), ("clk_cond", P32),
                ("never", ctypes.c_int32)]


class QueryDesc(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("p", PredDesc), ("q", PredDesc)]


class Stats(ctypes.Structure):
    _fields_ = [("explored", ctypes.c_uint64), ("generated", ctypes.c_uint64),
                ("expanded", ctypes.c_uint64), ("stored", ctypes.c_uint64),
                ("keys", ctypes.c_uint64), ("levels", ctypes.c_uint64), ("probes", ctypes.c_uint64),
                ("pre_calls", ctypes.c_uint64), ("gfp_iters", ctypes.c_uint64),
                ("kernel_launches", ctypes.c_uint64), ("seconds", ctypes.c_double),
                ("device_seconds", ctypes.c_double), ("extrapolating", ctypes.c_int32),
                ("status", ctypes.c_int32), ("kernel_seconds", ctypes.c_double * 6),
                ("kernel_calls", ctypes.c_uint64 * 6), ("h2d_bytes", ctypes.c_uint64),
                ("d2h_bytes", ctypes.c_uint64), ("probe_full", ctypes.c_uint64),
                ("merge_surv", ctypes.c_uint64), ("merge_live", ctypes.c_uint64), ("nodes", ctypes.c_uint64)]
    KERNELS = ("expand", "probe", "deadlock", "group", "merge", "other")

    def as_dict(self):
        d = {k: getattr(self, k) for k, _ in self._fields_ if k not in ("kernel_seconds", "kernel_calls")}
        d["kernel_seconds"] = {n: self.kernel_seconds[i] for i, n in enumerate(self.KERNELS)}
        d["kernel_calls"] = {n: int(self.kernel_calls[i]) for i, n in enumerate(self.KERNELS)}
        return d


def _i32(a) -> np.ndarray:
    a = np.ascontiguousarray(np.asarray(a, dtype=np.int32).reshape(-1))
    if a.size == 0:
        a = np.zeros(1, dtype=np.int32)   # never hand out a null pointer
    return a


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(P32)


class NetArrays:
    """Flattened arrays of a Network plus a NetDesc pointing into them (kept alive together)."""

    def __init__(self, net: Network):
        self.net = net
        cons: list = []
        iatoms: list = []
        resets: list = []
        iupds: list = []
        loc_flags, loc_inv_off = [], [0]
        for p in net.procs:
            for l in p.locations:
                loc_flags.append((LOC_URGENT if l.urgent else 0) | (LOC_COMMITTED if l.committed else 0))
                cons.extend(l.invariant)
                loc_inv_off.append(len(cons))
        e_proc, e_src, e_tgt, e_chan, e_dir = [], [], [], [], []
        g_off, ig_off, r_off, u_off = [len(cons)], [0], [0], [0]
        # edge guard offsets start after the invariants
        for pi, p in enumerate(net.procs):
            for e in p.edges:
                e_proc.append(pi); e_src.append(e.src); e_tgt.append(e.tgt)
                e_chan.append(e.chan); e_dir.append(e.dir)
                cons.extend(e.guard); g_off.append(len(cons))
                iatoms.extend(e.iguard); ig_off.append(len(iatoms))
                resets.extend(e.resets); r_off.append(len(resets))
                iupds.extend(e.iupd); u_off.append(len(iupds))
        self.arrays = {
            "chan_flags": _i32([f for _, f in net.chans]),
            "int_lo": _i32([v.lo for v in net.ints]), "int_hi": _i32([v.hi for v in net.ints]),
            "int_init": _i32([v.init for v in net.ints]),
            "proc_nlocs": _i32([len(p.locations) for p in net.procs]),
            "proc_init": _i32([p.initial for p in net.procs]),
            "loc_flags": _i32(loc_flags), "loc_inv_off": _i32(loc_inv_off),
            "edge_proc": _i32(e_proc), "edge_src": _i32(e_src), "edge_tgt": _i32(e_tgt),
            "edge_chan": _i32(e_chan), "edge_dir": _i32(e_dir),
            "edge_guard_off": _i32(g_off), "edge_iguard_off": _i32(ig_off),
            "edge_reset_off": _i32(r_off), "edge_iupd_off": _i32(u_off),
            "cons": _i32(cons), "iatoms": _i32(iatoms), "resets": _i32(resets), "iupds": _i32(iupds),
        }
        d = NetDesc()
        d.nclocks = net.nclocks
        d.nprocs = len(net.procs)
        d.nints = len(net.ints)
        d.nchans = len(net.chans)
        d.nedges = len(e_proc)
        for k, a in self.arrays.items():
            setattr(d, k, _ptr(a))
        self.desc = d

    @property
    def ref(self):
        return ctypes.byref(self.desc)


class PredArrays:
    def __init__(self, pred: Pred | None):
        pred = pred or Pred()
        self.pred = pred
        self.loc = _i32([x for lr in pred.loc_req for x in lr])
        self.int = _i32([x for a in pred.int_cond for x in a])
        self.clk = _i32([x for c in pred.clk_cond for x in c])
        d = PredDesc()
        d.nloc = len(pred.loc_req); d.loc_req = _ptr(self.loc)
        d.nint = len(pred.int_cond); d.int_cond = _ptr(self.int)
        d.nclk = len(pred.clk_cond); d.clk_cond = _ptr(self.clk)
        d.never = int(pred.never)
        self.desc = d

    @property
    def ref(self):
        return ctypes.byref(self.desc)


Q_REACH, Q_DEADLOCK, Q_LEADSTO, Q_EG = 0, 1, 2, 3


class QueryArrays:
    def __init__(self, kind: int, p: Pred | None = None, q: Pred | None = None):
        self.kind = kind
        self.pa = PredArrays(p)
        self.qa = PredArrays(q)
        d = QueryDesc()
        d.kind = kind
        d.p = self.pa.desc
        d.q = self.qa.desc
        self.desc = d


def query_from_json(d) -> Tuple[int, Pred, Pred]:
    return d["kind"], Pred.from_json(d["p"]), Pred.from_json(d["q"]) if d.get("q") else Pred()


def query_to_json(kind: int, p: Pred, q: Pred | None = None):
    return {"kind": kind, "p": p.to_json(), "q": (q or Pred()).to_json()}


def origin_zone(dim: int) -> np.ndarray:
    return np.full((dim, dim), ZERO_LE, dtype=np.int32)
