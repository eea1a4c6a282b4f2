"""Python face of the engine, mirroring the reference's query entry points.

Names and argument meanings follow include/hora/reachability.hpp (``reachable_net``),
include/hora/liveness.hpp (``deadlock_reachable``, ``leads_to_clocks``) and
include/hora/query.hpp (``check_network_query``). Every call goes through libhora_gb300.so; there
is no Python or CPU fallback, and a missing library or device raises.
"""
from __future__ import annotations

import ctypes
import enum
from dataclasses import dataclass, field
from typing import List, Optional, Sequence, Tuple

import numpy as np

from . import capi
from .model import (Network, Pred, NetArrays, PredArrays, QueryArrays, Stats, QueryDesc, NetDesc,
                    Q_REACH, Q_DEADLOCK, Q_LEADSTO, Q_EG)


class Backend(enum.IntEnum):
    """enum class Backend { Seq, Omp, Cuda, Metal } (include/hora/reach.hpp:21)."""
    Seq = 0
    Omp = 1
    Cuda = 2
    Metal = 3


@dataclass
class ReachStats:
    """ReachStats (include/hora/reach.hpp:10-19) plus the engine's own counters."""
    explored: int = 0
    generated: int = 0
    expanded: int = 0
    stored: int = 0
    keys: int = 0
    levels: int = 0
    probes: int = 0
    kernel_launches: int = 0
    seconds: float = 0.0
    device_seconds: float = 0.0
    extrapolating: bool = False
    status: int = 0
    h2d_bytes: int = 0
    d2h_bytes: int = 0
    probe_full: int = 0     # stored zones the probe read whole
    merge_surv: int = 0     # survivors folded by the merge
    merge_live: int = 0     # live zones of the merged keys before each merge
    nodes: int = 0          # zones written to the passed store
    pre_calls: int = 0      # exact predecessors of the backward sweep
    gfp_iters: int = 0      # rounds of the backward sweep
    kernels: dict = field(default_factory=dict)   # family -> {"seconds", "calls"}

    def fill(self, st: Stats):
        for k in ("explored", "generated", "expanded", "stored", "keys", "levels", "probes",
                  "kernel_launches", "seconds", "device_seconds", "status", "h2d_bytes", "d2h_bytes",
                  "probe_full", "merge_surv", "merge_live", "nodes", "pre_calls", "gfp_iters"):
            setattr(self, k, getattr(st, k))
        self.extrapolating = bool(st.extrapolating)
        self.kernels = {n: {"seconds": st.kernel_seconds[i], "calls": int(st.kernel_calls[i])}
                        for i, n in enumerate(Stats.KERNELS)}
        return self


def reachable_net(net: Network, target: Pred, backend: Backend = Backend.Cuda,
                  stats: Optional[ReachStats] = None) -> bool:
    """E<> target: is a symbolic state matching `target` reachable?"""
    L = capi.load()
    na, ta = NetArrays(net), PredArrays(target)
    st = Stats()
    res = ctypes.c_int32(0)
    rc = L.hora_gb_reachable_net(ctypes.addressof(na.desc), ctypes.addressof(ta.desc), int(backend),
                                 ctypes.byref(st), ctypes.byref(res))
    if stats is not None:
        stats.fill(st)
    capi.check(rc, "reachable_net")
    return bool(res.value)


def deadlock_reachable(net: Network, backend: Backend = Backend.Cuda, stats: Optional[ReachStats] = None,
                       cancel: Optional[ctypes.c_int32] = None) -> bool:
    """Is a state containing a deadlocked valuation reachable?  (A[] not deadlock == not this.)"""
    L = capi.load()
    na = NetArrays(net)
    st = Stats()
    res = ctypes.c_int32(0)
    rc = L.hora_gb_deadlock_reachable(ctypes.addressof(na.desc), int(backend), ctypes.byref(st),
                                      ctypes.byref(cancel) if cancel is not None else None, ctypes.byref(res))
    if stats is not None:
        stats.fill(st)
    capi.check(rc, "deadlock_reachable")
    return bool(res.value)


def leads_to_clocks(net: Network, p: Pred, q: Pred, backend: Backend = Backend.Cuda,
                    stats: Optional[ReachStats] = None) -> bool:
    """p --> q, both sides conjunctions that may carry clock atoms."""
    L = capi.load()
    na, pa, qa = NetArrays(net), PredArrays(p), PredArrays(q)
    st = Stats()
    res = ctypes.c_int32(0)
    rc = L.hora_gb_leads_to(ctypes.addressof(na.desc), ctypes.addressof(pa.desc), ctypes.addressof(qa.desc),
                            int(backend), ctypes.byref(st), ctypes.byref(res))
    if stats is not None:
        stats.fill(st)
    capi.check(rc, "leads_to")
    return bool(res.value)


def leads_to_otf(net: Network, p: Pred, q: Pred, backend: Backend = Backend.Cuda,
                 stats: Optional[ReachStats] = None) -> bool:
    """p --> q (leads_to_otf, include/hora/liveness.hpp:123-124): the same query and route as
    leads_to_clocks -- the reference's two entry points differ only in how they build their graph."""
    return leads_to_clocks(net, p, q, backend, stats)


def exists_invariant_run(net: Network, psi: Pred, backend: Backend = Backend.Cuda,
                         stats: Optional[ReachStats] = None) -> bool:
    """E[] psi (exists_invariant_run, include/hora/liveness.hpp:35-46): psi a conjunction of
    location (a negative location l stands for "not at -l-1"), integer and clock atoms."""
    L = capi.load()
    na, pa = NetArrays(net), PredArrays(psi)
    st = Stats()
    res = ctypes.c_int32(0)
    rc = L.hora_gb_exists_invariant(ctypes.addressof(na.desc), ctypes.addressof(pa.desc), int(backend),
                                    ctypes.byref(st), ctypes.byref(res))
    if stats is not None:
        stats.fill(st)
    capi.check(rc, "exists_invariant")
    return bool(res.value)


def exists_invariant_trace(net: Network, psi: Pred, backend: Backend = Backend.Cuda, cap: int = 1 << 16):
    """E[] psi with a witness: (holds, trace) where trace = dict(ords, locs, ints, zones, loop_to,
    loop_ord) or None when psi fails (see hora_gb_exists_invariant_trace)."""
    L = capi.load()
    na, pa = NetArrays(net), PredArrays(psi)
    np_, ni, d2 = len(net.procs), len(net.ints), net.dim * net.dim
    st = Stats()
    res, n, lt, lo = ctypes.c_int32(0), ctypes.c_int32(0), ctypes.c_int32(0), ctypes.c_int32(0)
    ords = np.zeros(max(cap, 1), np.int32)
    locs = np.zeros(max(cap * np_, 1), np.int32)
    ints = np.zeros(max(cap * ni, 1), np.int32)
    zones = np.zeros(max(cap * d2, 1), np.int32)
    rc = L.hora_gb_exists_invariant_trace(ctypes.addressof(na.desc), ctypes.addressof(pa.desc), int(backend),
                                          ctypes.byref(st), ctypes.byref(res), cap, ctypes.byref(n),
                                          capi.p32(ords), capi.p32(locs), capi.p32(ints), capi.p32(zones),
                                          ctypes.byref(lt), ctypes.byref(lo))
    capi.check(rc, "exists_invariant_trace")
    k = n.value
    if not res.value or k == 0:
        return bool(res.value), None
    return True, {"ords": ords[:k].tolist(), "locs": locs[:k * np_].reshape(k, np_),
                  "ints": ints[:k * ni].reshape(k, ni), "zones": zones[:k * d2].reshape(k, net.dim, net.dim),
                  "loop_to": lt.value, "loop_ord": lo.value}


class QueryHandle:
    """One (network, query) pair opened once and run on demand (hora_gb_open / hora_gb_run /
    hora_gb_trace / hora_gb_close); usable as a context manager. ``kind`` and the predicates follow
    ``check_network_query`` without ``negate``: run() returns reachable (Q_REACH), deadlock
    reachable (Q_DEADLOCK), holds (Q_LEADSTO, Q_EG)."""

    def __init__(self, net: Network, kind: int, p: Optional[Pred] = None, q: Optional[Pred] = None):
        self._lib = capi.load()
        self.net, self.kind = net, kind
        na, qa = NetArrays(net), QueryArrays(kind, p or Pred(), q or Pred())
        h = ctypes.c_void_p()
        capi.check(self._lib.hora_gb_open(ctypes.addressof(na.desc), ctypes.addressof(qa.desc), ctypes.byref(h)),
                   "open")
        self._h = h   # the library copied the descriptors

    def run(self, stats: Optional[ReachStats] = None) -> bool:
        st = Stats()
        v = ctypes.c_int32(-1)
        rc = self._lib.hora_gb_run(self._h, ctypes.byref(v), ctypes.byref(st))
        if stats is not None:
            stats.fill(st)
        capi.check(rc, "run")
        return bool(v.value)

    def trace(self, cap: int = 1 << 16):
        """The trace of the last run (hora_gb_trace): the witness of an E[] query (as
        exists_invariant_trace); for reach / deadlock / a leads-to violation found by the early
        witness, the counterexample path from the initial state to the goal, ords[i] the transition
        index of step i; for a leads-to violation found by the backward sweep, the path to a p-state,
        the root cut from it (ords -2), then a path of the !q graph to a stop set or around a cycle
        (loop_to, loop_ord). None when there is none."""
        net = self.net
        np_, ni, d2 = len(net.procs), len(net.ints), net.dim * net.dim
        n, lt, lo = ctypes.c_int32(0), ctypes.c_int32(0), ctypes.c_int32(0)
        ords = np.zeros(max(cap, 1), np.int32)
        locs = np.zeros(max(cap * np_, 1), np.int32)
        ints = np.zeros(max(cap * ni, 1), np.int32)
        zones = np.zeros(max(cap * d2, 1), np.int32)
        rc = self._lib.hora_gb_trace(self._h, cap, ctypes.byref(n), capi.p32(ords), capi.p32(locs), capi.p32(ints),
                                     capi.p32(zones), ctypes.byref(lt), ctypes.byref(lo))
        capi.check(rc, "trace")
        k = n.value
        if k == 0:
            return None
        return {"ords": ords[:k].tolist(), "locs": locs[:k * np_].reshape(k, np_),
                "ints": ints[:k * ni].reshape(k, ni), "zones": zones[:k * d2].reshape(k, net.dim, net.dim),
                "loop_to": lt.value, "loop_ord": lo.value}

    def close(self):
        if self._h:
            capi.check(self._lib.hora_gb_close(self._h), "close")
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        if getattr(self, "_h", None):
            try:
                self._lib.hora_gb_close(self._h)
            except Exception:   # interpreter shutdown: the library may already be gone
                pass
            self._h = None


def check_network_query(net: Network, kind: int, p: Pred, q: Optional[Pred] = None, negate: bool = False,
                        backend: Backend = Backend.Cuda, stats: Optional[ReachStats] = None) -> bool:
    """Route one lowered query (check_network_query, src/query/dispatch.cpp:109-607).

    ``kind`` is Q_REACH (E<> p; ``negate`` gives A[] not p), Q_DEADLOCK (``negate`` gives
    A[] not deadlock), Q_LEADSTO (p --> q) or Q_EG (E[] p; ``negate`` with p = not phi gives
    A<> phi). Returns whether the formula is satisfied.
    """
    if kind == Q_REACH:
        r = reachable_net(net, p, backend, stats)
    elif kind == Q_DEADLOCK:
        r = deadlock_reachable(net, backend, stats)
    elif kind == Q_LEADSTO:
        r = leads_to_clocks(net, p, q or Pred(), backend, stats)
    elif kind == Q_EG:
        r = exists_invariant_run(net, p, backend, stats)
    else:
        raise ValueError(kind)
    return (not r) if negate else r


def expand(net: Network, locs, ints, zones, L, U, qmask=None, emode: int = 0, cap: Optional[int] = None):
    """Successor pipeline on explicit states (hora_gb_expand): dict of arrays in emission order."""
    lib = capi.load()
    na = NetArrays(net)
    dim, np_, ni = net.dim, len(net.procs), len(net.ints)
    locs = np.ascontiguousarray(locs, np.int32).reshape(-1, np_)
    n = locs.shape[0]
    ints = np.ascontiguousarray(ints, np.int32).reshape(n, ni) if ni else np.zeros((n, 1), np.int32)
    zones = np.ascontiguousarray(zones, np.int32).reshape(n, dim, dim)
    L = np.ascontiguousarray(L, np.int32)
    U = np.ascontiguousarray(U, np.int32)
    qm = np.zeros(dim, np.uint8) if qmask is None else np.ascontiguousarray(qmask, np.uint8)
    cap = cap or max(16, n * 64)
    while True:
        o_src = np.zeros(cap, np.int32); o_ord = np.zeros(cap, np.int32)
        o_locs = np.zeros((cap, np_), np.int32); o_ints = np.zeros((cap, max(ni, 1)), np.int32)
        o_z = np.zeros((cap, dim, dim), np.int32)
        out_n = ctypes.c_int64(0)
        rc = lib.hora_gb_expand(ctypes.addressof(na.desc), n, capi.p32(locs), capi.p32(ints), capi.p32(zones),
                                capi.p32(L), capi.p32(U), qm.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)), emode,
                                cap, capi.p32(o_src), capi.p32(o_ord), capi.p32(o_locs), capi.p32(o_ints),
                                capi.p32(o_z), ctypes.byref(out_n))
        if rc == capi.E_OVERFLOW:
            cap = int(out_n.value)
            continue
        capi.check(rc, "expand")
        k = int(out_n.value)
        return {"src": o_src[:k], "ord": o_ord[:k], "locs": o_locs[:k], "ints": o_ints[:k, :ni], "zones": o_z[:k]}


def has_deadlock(net: Network, locs, ints, zones) -> np.ndarray:
    lib = capi.load()
    na = NetArrays(net)
    dim, np_, ni = net.dim, len(net.procs), len(net.ints)
    locs = np.ascontiguousarray(locs, np.int32).reshape(-1, np_)
    n = locs.shape[0]
    ints = np.ascontiguousarray(ints, np.int32).reshape(n, ni) if ni else np.zeros((n, 1), np.int32)
    zones = np.ascontiguousarray(zones, np.int32).reshape(n, dim, dim)
    out = np.zeros(n, np.int32)
    rc = lib.hora_gb_has_deadlock(ctypes.addressof(na.desc), n, capi.p32(locs), capi.p32(ints), capi.p32(zones),
                                  capi.p32(out))
    capi.check(rc, "has_deadlock")
    return out.astype(bool)


class BatchInput:
    """The descriptors of a batch, built once (their arrays stay alive with this object)."""

    def __init__(self, items: Sequence[Tuple[Network, int, Pred, Pred]]):
        self.n = len(items)
        self.nas = [NetArrays(it[0]) for it in items]
        self.qas = [QueryArrays(it[1], it[2], it[3]) for it in items]
        self.nets = (NetDesc * max(self.n, 1))(*[a.desc for a in self.nas])
        self.qs = (QueryDesc * max(self.n, 1))(*[a.desc for a in self.qas])


def batch_run(items, cancel: Optional[ctypes.c_int32] = None):
    """Run (network, kind, p, q) instances together; returns (verdicts, [stats dict]). `items` is a
    sequence of tuples or a prepared BatchInput.

    cancel: a ctypes.c_int32 another thread may set to 1; instances without a verdict by then come
    back with verdict -1 and stats status E_CANCELLED (no exception is raised for that)."""
    lib = capi.load()
    b = items if isinstance(items, BatchInput) else BatchInput(items)
    n, nets, qs = b.n, b.nets, b.qs
    verdicts = np.zeros(max(n, 1), np.int32)
    stats = (Stats * max(n, 1))()
    rc = lib.hora_gb_batch_run(n, ctypes.addressof(nets), ctypes.addressof(qs), capi.p32(verdicts),
                               ctypes.addressof(stats), ctypes.addressof(cancel) if cancel is not None else None)
    if rc != capi.E_CANCELLED:
        capi.check(rc, "batch_run")
    return verdicts[:n].tolist(), [stats[k].as_dict() for k in range(n)]


class Server:
    """The serving form (hora_gb_server_*): requests are queued and admitted in arrival order while
    at most `max_inflight` run and the `budget_bytes` pool holds their initial store reservation;
    each runs on its own worker and stream, its stores growing from the pool level by level.
    `per_request_bytes` (0: none) bounds one request's store -- past it the request stops with
    HORA_E_BUDGET; `max_queued` (0: none) rejects a submission that finds that many requests waiting.
    `poll` returns (verdict, stats dict) once a ticket is done (the result is then released), else
    None; closing cancels what still runs."""

    def __init__(self, budget_bytes: int, max_inflight: int, per_request_bytes: int = 0, max_queued: int = 0):
        self._lib = capi.load()
        self._h = ctypes.c_void_p()
        capi.check(self._lib.hora_gb_server_create(int(budget_bytes), int(max_inflight), ctypes.byref(self._h)),
                   "server_create")
        if per_request_bytes or max_queued:
            capi.check(self._lib.hora_gb_server_set_limits(self._h, int(per_request_bytes), int(max_queued)),
                       "server_set_limits")

    def submit(self, net: Network, kind: int, p: Pred, q: Optional[Pred] = None) -> int:
        na, qa = NetArrays(net), QueryArrays(kind, p, q)
        t = ctypes.c_int64(0)
        capi.check(self._lib.hora_gb_server_submit(self._h, ctypes.addressof(na.desc), ctypes.addressof(qa.desc),
                                                   ctypes.byref(t)), "server_submit")
        return t.value   # the descriptors were copied: na/qa may go

    def active(self) -> int:
        a = ctypes.c_int32(0)
        capi.check(self._lib.hora_gb_server_step(self._h, ctypes.byref(a)), "server_step")
        return a.value

    def poll(self, ticket: int):
        d, v, st = ctypes.c_int32(0), ctypes.c_int32(0), Stats()
        capi.check(self._lib.hora_gb_server_poll(self._h, ticket, ctypes.byref(d), ctypes.byref(v),
                                                 ctypes.byref(st)), "server_poll")
        return (v.value, st.as_dict()) if d.value else None

    def drain(self, timeout: float = 600.0):
        import time
        t0 = time.perf_counter()
        while self.active() > 0:
            if time.perf_counter() - t0 > timeout:
                raise TimeoutError("server did not drain")

    def close(self):
        if self._h:
            capi.check(self._lib.hora_gb_server_destroy(self._h), "server_destroy")
            self._h = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
