"""ctypes binding of the CPU oracle (oracle/hora_oracle.c).  TEST INFRASTRUCTURE ONLY.

Loaded only by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg, as the checker of
the CUDA engine. The product package (ptctcl_gb300) never imports this module.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

from ptctcl_gb300.model import (NetArrays, PredArrays, Stats, Network, Pred, P32)

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libhora_oracle.so")
_lib = None


def build(force: bool = False) -> str:
    if force or not os.path.exists(_LIB_PATH) or (
            os.path.getmtime(_LIB_PATH) < max(os.path.getmtime(os.path.join(_HERE, f))
                                                for f in ("hora_oracle.c", "hora_oracle.h"))):
        subprocess.check_call(["make", "-s", "-C", _HERE])
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build())
        L = _lib
        I32, I64 = ctypes.c_int32, ctypes.c_int64
        VP = ctypes.c_void_p
        for name in ("orc_dbm_init", "orc_dbm_close", "orc_dbm_delay", "orc_dbm_down"):
            getattr(L, name).argtypes = [P32, I32]
            getattr(L, name).restype = None
        L.orc_dbm_empty.argtypes = [P32, I32]; L.orc_dbm_empty.restype = I32
        L.orc_dbm_constrain.argtypes = [P32, I32, I32, I32, I32]; L.orc_dbm_constrain.restype = I32
        L.orc_dbm_reset.argtypes = [P32, I32, I32]; L.orc_dbm_reset.restype = None
        L.orc_dbm_free.argtypes = [P32, I32, I32]; L.orc_dbm_free.restype = None
        L.orc_dbm_includes.argtypes = [P32, P32, I32]; L.orc_dbm_includes.restype = I32
        L.orc_dbm_alu_le.argtypes = [P32, P32, I32, P32, P32]; L.orc_dbm_alu_le.restype = I32
        L.orc_dbm_extrap_lu_plus.argtypes = [P32, I32, P32, P32]; L.orc_dbm_extrap_lu_plus.restype = None
        L.orc_dbm_try_union.argtypes = [P32, P32, I32]; L.orc_dbm_try_union.restype = I32
        L.orc_fed_covers.argtypes = [P32, P32, I32, I32]; L.orc_fed_covers.restype = I32
        L.orc_static_bounds.argtypes = [VP, P32, P32, P32, P32, ctypes.POINTER(ctypes.c_uint64)]
        L.orc_static_bounds.restype = I32
        L.orc_expand.argtypes = [VP, I32, P32, P32, P32, P32, P32, ctypes.POINTER(ctypes.c_uint8), I32,
                                 I64, P32, P32, P32, P32, P32, ctypes.POINTER(I64)]
        L.orc_expand.restype = I32
        L.orc_has_deadlock.argtypes = [VP, I32, P32, P32, P32, P32]; L.orc_has_deadlock.restype = I32
        L.orc_reachable_net.argtypes = [VP, VP, VP, P32]; L.orc_reachable_net.restype = I32
        L.orc_deadlock_reachable.argtypes = [VP, VP, P32]; L.orc_deadlock_reachable.restype = I32
        L.orc_leads_to.argtypes = [VP, VP, VP, VP, P32]; L.orc_leads_to.restype = I32
        L.orc_exists_invariant.argtypes = [VP, VP, VP, P32]; L.orc_exists_invariant.restype = I32
        L.orc_eg_initial.argtypes = [VP, VP, P32, P32, P32]; L.orc_eg_initial.restype = I32
        L.orc_eg_successors.argtypes = [VP, VP, P32, P32, P32, I32, P32, P32, P32, P32]
        L.orc_eg_successors.restype = I32
        L.orc_initial_state.argtypes = [VP, ctypes.POINTER(ctypes.c_uint8), P32, P32, P32]
        L.orc_initial_state.restype = I32
        L.orc_set_time_limit.argtypes = [ctypes.c_double]
        L.orc_set_time_limit.restype = None
        L.orc_successor_raw.argtypes = [VP, ctypes.POINTER(ctypes.c_uint8), P32, P32, P32, I32, P32, P32, P32]
        L.orc_successor_raw.restype = I32
        L.orc_lt_successor_raw.argtypes = [VP, VP, ctypes.POINTER(ctypes.c_uint8), P32, P32, P32, I32, P32, P32, P32]
        L.orc_lt_successor_raw.restype = I32
        L.orc_lt_stop.argtypes = [VP, VP, ctypes.POINTER(ctypes.c_uint8), P32, P32, P32]
        L.orc_lt_stop.restype = I32
        L.orc_set_threads.argtypes = [I32]
        L.orc_set_threads.restype = I32
    return _lib


def set_time_limit(seconds: float):
    lib().orc_set_time_limit(float(seconds))


def set_threads(n: int) -> int:
    """Host threads of the E<> / deadlock reachability route; returns the count in effect."""
    return int(lib().orc_set_threads(int(n)))


def _p(a: np.ndarray):
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(P32)


# ---- DBM primitives on numpy (dim x dim int32) ---------------------------------------------
class Dbm:
    """Thin numpy wrapper over the oracle's DBM primitives (the reference's hdbm::Dbm API)."""

    def __init__(self, nclocks: int = 0, data=None):
        if data is not None:
            self.d = np.ascontiguousarray(np.array(data, dtype=np.int32))
        else:
            self.d = np.zeros((nclocks + 1, nclocks + 1), dtype=np.int32)
            lib().orc_dbm_init(_p(self.d), nclocks + 1)

    @property
    def dim(self):
        return self.d.shape[0]

    def copy(self):
        return Dbm(data=self.d.copy())

    def get(self, i, j):
        return int(self.d[i, j])

    def empty(self):
        return bool(lib().orc_dbm_empty(_p(self.d), self.dim))

    def close(self):
        lib().orc_dbm_close(_p(self.d), self.dim); return self

    def constrain(self, i, j, raw):
        return bool(lib().orc_dbm_constrain(_p(self.d), self.dim, i, j, raw))

    def reset(self, k):
        lib().orc_dbm_reset(_p(self.d), self.dim, k); return self

    def delay(self):
        lib().orc_dbm_delay(_p(self.d), self.dim); return self

    def down(self):
        lib().orc_dbm_down(_p(self.d), self.dim); return self

    def free(self, k):
        lib().orc_dbm_free(_p(self.d), self.dim, k); return self

    def includes(self, other: "Dbm"):
        return bool(lib().orc_dbm_includes(_p(self.d), _p(other.d), self.dim))

    def alu_le(self, other: "Dbm", L, U):
        L = np.ascontiguousarray(L, dtype=np.int32); U = np.ascontiguousarray(U, dtype=np.int32)
        return bool(lib().orc_dbm_alu_le(_p(self.d), _p(other.d), self.dim, _p(L), _p(U)))

    def extrapolate_lu_plus(self, L, U):
        L = np.ascontiguousarray(L, dtype=np.int32); U = np.ascontiguousarray(U, dtype=np.int32)
        lib().orc_dbm_extrap_lu_plus(_p(self.d), self.dim, _p(L), _p(U)); return self

    def try_union(self, other: "Dbm"):
        return bool(lib().orc_dbm_try_union(_p(self.d), _p(other.d), self.dim))


def fed_covers(z: Dbm, ws) -> bool:
    w = np.ascontiguousarray(np.stack([x.d for x in ws]) if ws else np.zeros((1, z.dim, z.dim), np.int32))
    return bool(lib().orc_fed_covers(_p(z.d), _p(w), len(ws), z.dim))


# ---- model-level calls ------------------------------------------------------------------------
def static_bounds(net: Network):
    na = NetArrays(net)
    dim = net.dim
    nl = sum(len(p.locations) for p in net.procs)
    L = np.zeros(dim, np.int32); U = np.zeros(dim, np.int32)
    Ll = np.zeros(nl * dim, np.int32); Ul = np.zeros(nl * dim, np.int32)
    act = np.zeros(nl, np.uint64)
    rc = lib().orc_static_bounds(ctypes.addressof(na.desc), _p(L), _p(U), _p(Ll), _p(Ul),
                                 act.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)))
    assert rc == 0, rc
    return L, U, Ll.reshape(nl, dim), Ul.reshape(nl, dim), act


def expand(net: Network, locs, ints, zones, L, U, qmask=None, emode=0, cap=None):
    """Successors of n states in (source, emission) order: returns dict of arrays."""
    na = NetArrays(net)
    dim, np_, ni = net.dim, len(net.procs), len(net.ints)
    locs = np.ascontiguousarray(locs, np.int32).reshape(-1, np_)
    n = locs.shape[0]
    ints = np.ascontiguousarray(ints, np.int32).reshape(n, ni) if ni else np.zeros((n, 1), np.int32)
    zones = np.ascontiguousarray(zones, np.int32).reshape(n, dim, dim)
    L = np.ascontiguousarray(L, np.int32); U = np.ascontiguousarray(U, np.int32)
    qm = np.zeros(dim, np.uint8) if qmask is None else np.ascontiguousarray(qmask, np.uint8)
    cap = cap or max(16, n * 64)
    while True:
        o_src = np.zeros(cap, np.int32); o_ord = np.zeros(cap, np.int32)
        o_locs = np.zeros((cap, np_), np.int32); o_ints = np.zeros((cap, max(ni, 1)), np.int32)
        o_z = np.zeros((cap, dim, dim), np.int32)
        out_n = ctypes.c_int64(0)
        rc = lib().orc_expand(ctypes.addressof(na.desc), n, _p(locs), _p(ints), _p(zones), _p(L), _p(U),
                              qm.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)), emode, cap,
                              _p(o_src), _p(o_ord), _p(o_locs), _p(o_ints), _p(o_z), ctypes.byref(out_n))
        if rc == 4:
            cap = int(out_n.value)
            continue
        assert rc == 0, rc
        k = int(out_n.value)
        return {"src": o_src[:k], "ord": o_ord[:k], "locs": o_locs[:k], "ints": o_ints[:k, :ni],
                "zones": o_z[:k]}


def has_deadlock(net: Network, locs, ints, zones):
    na = NetArrays(net)
    dim, np_, ni = net.dim, len(net.procs), len(net.ints)
    locs = np.ascontiguousarray(locs, np.int32).reshape(-1, np_)
    n = locs.shape[0]
    ints = np.ascontiguousarray(ints, np.int32).reshape(n, ni) if ni else np.zeros((n, 1), np.int32)
    zones = np.ascontiguousarray(zones, np.int32).reshape(n, dim, dim)
    out = np.zeros(n, np.int32)
    rc = lib().orc_has_deadlock(ctypes.addressof(na.desc), n, _p(locs), _p(ints), _p(zones), _p(out))
    assert rc == 0, rc
    return out.astype(bool)


def successor_raw(net: Network, locs, ints, zone, raw: int, qmask=None):
    """The exact successor by transition index `raw`, or None when that transition yields nothing."""
    na = NetArrays(net)
    np_, ni, d = len(net.procs), len(net.ints), net.dim
    l = np.ascontiguousarray(locs, np.int32).reshape(-1)
    i = np.ascontiguousarray(ints, np.int32).reshape(-1) if ni else np.zeros(1, np.int32)
    z = np.ascontiguousarray(zone, np.int32).reshape(-1)
    qm = np.zeros(64, np.uint8)
    if qmask is not None:
        qm[:len(qmask)] = np.asarray(qmask, np.uint8)
    ol, oi, oz = np.zeros(max(np_, 1), np.int32), np.zeros(max(ni, 1), np.int32), np.zeros(d * d, np.int32)
    ok = lib().orc_successor_raw(ctypes.addressof(na.desc), qm.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)),
                                 _p(l), _p(i), _p(z), int(raw), _p(ol), _p(oi), _p(oz))
    if not ok:
        return None
    return ol[:np_], oi[:ni], oz.reshape(d, d)


def lt_successor_raw(net: Network, q: Pred, locs, ints, zone, raw: int, qmask=None):
    """Leads-to phase 2: the successor by transition index `raw` in the network restricted to !q
    (!q adjoined to the invariants), or None when that transition yields nothing."""
    na, qa = NetArrays(net), PredArrays(q)
    np_, ni, d = len(net.procs), len(net.ints), net.dim
    l = np.ascontiguousarray(locs, np.int32).reshape(-1)
    i = np.ascontiguousarray(ints, np.int32).reshape(-1) if ni else np.zeros(1, np.int32)
    z = np.ascontiguousarray(zone, np.int32).reshape(-1)
    qm = np.zeros(64, np.uint8)
    if qmask is not None:
        qm[:len(qmask)] = np.asarray(qmask, np.uint8)
    ol, oi, oz = np.zeros(max(np_, 1), np.int32), np.zeros(max(ni, 1), np.int32), np.zeros(d * d, np.int32)
    ok = lib().orc_lt_successor_raw(ctypes.addressof(na.desc), ctypes.addressof(qa.desc),
                                    qm.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)),
                                    _p(l), _p(i), _p(z), int(raw), _p(ol), _p(oi), _p(oz))
    if not ok:
        return None
    return ol[:np_], oi[:ni], oz.reshape(d, d)


def lt_stop(net: Network, q: Pred, locs, ints, zone, qmask=None) -> int:
    """Leads-to phase 2: the stop set of a state's zone -- 0 empty, 1 its deadlocked valuations,
    2 the whole zone."""
    na, qa = NetArrays(net), PredArrays(q)
    ni = len(net.ints)
    l = np.ascontiguousarray(locs, np.int32).reshape(-1)
    i = np.ascontiguousarray(ints, np.int32).reshape(-1) if ni else np.zeros(1, np.int32)
    z = np.ascontiguousarray(zone, np.int32).reshape(-1)
    qm = np.zeros(64, np.uint8)
    if qmask is not None:
        qm[:len(qmask)] = np.asarray(qmask, np.uint8)
    return int(lib().orc_lt_stop(ctypes.addressof(na.desc), ctypes.addressof(qa.desc),
                                 qm.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)), _p(l), _p(i), _p(z)))


def initial_state(net: Network, qmask=None):
    na = NetArrays(net)
    dim = net.dim
    qm = np.zeros(dim, np.uint8) if qmask is None else np.ascontiguousarray(qmask, np.uint8)
    locs = np.zeros(len(net.procs), np.int32); ints = np.zeros(max(1, len(net.ints)), np.int32)
    z = np.zeros((dim, dim), np.int32)
    ok = lib().orc_initial_state(ctypes.addressof(na.desc), qm.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)),
                                 _p(locs), _p(ints), _p(z))
    return bool(ok), locs, ints[:len(net.ints)], z


def reachable_net(net: Network, target: Pred):
    na, ta = NetArrays(net), PredArrays(target)
    st = Stats(); res = ctypes.c_int32(0)
    rc = lib().orc_reachable_net(ctypes.addressof(na.desc), ctypes.addressof(ta.desc), ctypes.byref(st),
                                 ctypes.byref(res))
    if rc:
        raise RuntimeError(f"oracle reachable_net status {rc}")
    return bool(res.value), st.as_dict()


def deadlock_reachable(net: Network):
    na = NetArrays(net)
    st = Stats(); res = ctypes.c_int32(0)
    rc = lib().orc_deadlock_reachable(ctypes.addressof(na.desc), ctypes.byref(st), ctypes.byref(res))
    if rc or st.status not in (0, 5):
        raise RuntimeError(f"oracle deadlock_reachable status {rc}")
    return bool(res.value), st.as_dict()


def exists_invariant(net: Network, psi: Pred):
    """E[] psi from the initial state (psi a conjunction)."""
    na, pa = NetArrays(net), PredArrays(psi)
    st = Stats(); res = ctypes.c_int32(0)
    rc = lib().orc_exists_invariant(ctypes.addressof(na.desc), ctypes.addressof(pa.desc), ctypes.byref(st),
                                    ctypes.byref(res))
    if rc or st.status not in (0, 5):
        raise RuntimeError(f"oracle exists_invariant status {rc}")
    return bool(res.value), st.as_dict()


def eg_initial(net: Network, psi: Pred):
    """The psi-restricted initial state (locs, ints, zone), or None."""
    na, pa = NetArrays(net), PredArrays(psi)
    locs = np.zeros(max(len(net.procs), 1), np.int32)
    ints = np.zeros(max(len(net.ints), 1), np.int32)
    zone = np.zeros(net.dim * net.dim, np.int32)
    ok = lib().orc_eg_initial(ctypes.addressof(na.desc), ctypes.addressof(pa.desc), _p(locs), _p(ints), _p(zone))
    return (locs[:len(net.procs)], ints[:len(net.ints)], zone.reshape(net.dim, net.dim)) if ok else None


def eg_successors(net: Network, psi: Pred, locs, ints, zone):
    """Successors of one state in the psi-restricted graph, in emission order: (locs, ints, zones)."""
    na, pa = NetArrays(net), PredArrays(psi)
    np_, ni, d2 = len(net.procs), len(net.ints), net.dim * net.dim
    l = np.ascontiguousarray(locs, np.int32).reshape(-1)
    i = np.ascontiguousarray(ints, np.int32).reshape(-1) if ni else np.zeros(1, np.int32)
    z = np.ascontiguousarray(zone, np.int32).reshape(-1)
    cap = 4096
    ol, oi, oz = np.zeros(cap * max(np_, 1), np.int32), np.zeros(cap * max(ni, 1), np.int32), np.zeros(cap * d2, np.int32)
    n = ctypes.c_int32(0)
    rc = lib().orc_eg_successors(ctypes.addressof(na.desc), ctypes.addressof(pa.desc), _p(l), _p(i), _p(z), cap,
                                 _p(ol), _p(oi), _p(oz), ctypes.byref(n))
    if rc or n.value > cap:
        raise RuntimeError(f"oracle eg_successors status {rc}")
    k = n.value
    return ol[:k * np_].reshape(k, np_), oi[:k * ni].reshape(k, ni), oz[:k * d2].reshape(k, net.dim, net.dim)


def leads_to(net: Network, p: Pred, q: Pred):
    na, pa, qa = NetArrays(net), PredArrays(p), PredArrays(q)
    st = Stats(); res = ctypes.c_int32(0)
    rc = lib().orc_leads_to(ctypes.addressof(na.desc), ctypes.addressof(pa.desc), ctypes.addressof(qa.desc),
                            ctypes.byref(st), ctypes.byref(res))
    if rc or st.status not in (0, 5):
        raise RuntimeError(f"oracle leads_to status {rc}")
    return bool(res.value), st.as_dict()
