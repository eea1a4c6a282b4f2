"""CPU-side checks of the C ABI: the library loads, exports every declared entry point, and rejects
bad or out-of-scope input before touching a device."""
import ctypes
import os
import re

import pytest

from ptctcl_gb300 import capi
from ptctcl_gb300.model import NetArrays, PredArrays, Stats, Pred, Network, Process, Location, Edge, c_le
from golden_util import load_model

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    syms = set()
    for f in os.listdir(os.path.join(ROOT, "include")):
        if f.endswith(".h"):
            syms |= set(re.findall(r"HORA_GB_API\s+[\w\s\*]+?\b(hora_gb_\w+)\s*\(", open(os.path.join(ROOT, "include", f)).read()))
    return syms


def test_library_exports_every_declared_symbol():
    lib = capi.load()
    syms = declared_symbols()
    assert syms >= set(capi.EXPORTS)
    for s in syms:
        assert hasattr(lib, s), s
    assert lib.hora_gb_abi_version() == 2


def test_invalid_and_unsupported_inputs_are_rejected_without_a_device():
    lib = capi.load()
    res = ctypes.c_int32(7)
    st = Stats()
    # backend other than CUDA: the caller keeps its own engine
    net = load_model("fischer4")
    na, ta = NetArrays(net), PredArrays(Pred([(0, 3)]))
    rc = lib.hora_gb_reachable_net(ctypes.addressof(na.desc), ctypes.addressof(ta.desc), capi.BACKEND_OMP,
                                   ctypes.byref(st), ctypes.byref(res))
    assert rc == capi.E_NOT_SUPPORTED
    # diagonal constraint: out of scope, like the reference's CUDA factory
    diag = Network(2, [Process("P", [Location("A", [(1, 2, (3 << 1) | 1)])], [], 0)])
    na2 = NetArrays(diag)
    rc = lib.hora_gb_reachable_net(ctypes.addressof(na2.desc), ctypes.addressof(ta.desc), capi.BACKEND_CUDA,
                                   ctypes.byref(st), ctypes.byref(res))
    assert rc == capi.E_NOT_SUPPORTED and "diagonal" in capi.last_error()
    # target location out of range
    bad = PredArrays(Pred([(0, 99)]))
    rc = lib.hora_gb_reachable_net(ctypes.addressof(na.desc), ctypes.addressof(bad.desc), capi.BACKEND_CUDA,
                                   ctypes.byref(st), ctypes.byref(res))
    assert rc == capi.E_INVALID
    # more than 16 clocks
    wide = Network(17, [Process("P", [Location("A", [c_le(17, 3)])], [], 0)])
    na3 = NetArrays(wide)
    rc = lib.hora_gb_deadlock_reachable(ctypes.addressof(na3.desc), capi.BACKEND_CUDA, ctypes.byref(st), None,
                                        ctypes.byref(res))
    assert rc == capi.E_NOT_SUPPORTED
    # the serving form's limits need a server
    assert lib.hora_gb_server_set_limits(None, 1 << 30, 4) == capi.E_INVALID
    # the tuning table holds at most one entry per DBM dimension (0..17); it touches no device
    assert lib.hora_gb_set_tuning(None, None, None, 19) == capi.E_INVALID
    assert lib.hora_gb_set_tuning(None, None, None, 0) == capi.OK
    capi.set_tuning({"long_list": {9: 0, "7": 16}, "group_max": {9: 32}, "blocks_per_sm": {9: 8}})
    capi.set_tuning({})
    capi.apply_tuning()


@pytest.mark.skipif(capi.device_count() > 0, reason="needs a machine without a CUDA device")
def test_no_device_is_an_error_not_a_fallback():
    lib = capi.load()
    net = load_model("fischer4")
    na, ta = NetArrays(net), PredArrays(Pred([(0, 3)]))
    res = ctypes.c_int32(0)
    rc = lib.hora_gb_reachable_net(ctypes.addressof(na.desc), ctypes.addressof(ta.desc), capi.BACKEND_CUDA, None,
                                   ctypes.byref(res))
    assert rc == capi.E_NO_DEVICE


def test_handle_open_validates_and_copies_without_a_device():
    from ptctcl_gb300.model import QueryArrays
    lib = capi.load()
    net = load_model("fischer4")
    na = NetArrays(net)
    h = ctypes.c_void_p()

    def open_(kind, p, q=None):
        qa = QueryArrays(kind, p, q)
        return lib.hora_gb_open(ctypes.addressof(na.desc), ctypes.addressof(qa.desc), ctypes.byref(h))

    assert open_(0, Pred([(0, 3)])) == capi.OK and h.value
    n, lt, lo = ctypes.c_int32(0), ctypes.c_int32(0), ctypes.c_int32(0)
    rc = lib.hora_gb_trace(h, 0, ctypes.byref(n), None, None, None, None, ctypes.byref(lt), ctypes.byref(lo))
    assert rc == capi.E_INVALID and "not run" in capi.last_error()   # every kind keeps a trace once run
    assert lib.hora_gb_close(h) == capi.OK
    assert open_(3, Pred([(0, 3)])) == capi.OK
    rc = lib.hora_gb_trace(h, 0, ctypes.byref(n), None, None, None, None, ctypes.byref(lt), ctypes.byref(lo))
    assert rc == capi.E_INVALID   # not run yet
    assert lib.hora_gb_close(h) == capi.OK
    assert open_(0, Pred([(0, 99)])) == capi.E_INVALID and not h.value
    assert open_(7, Pred([(0, 3)])) == capi.E_INVALID
    diag = NetArrays(Network(2, [Process("P", [Location("A", [(1, 2, (3 << 1) | 1)])], [], 0)]))
    qa = QueryArrays(1, None, None)
    assert lib.hora_gb_open(ctypes.addressof(diag.desc), ctypes.addressof(qa.desc), ctypes.byref(h)) == \
        capi.E_NOT_SUPPORTED
    assert lib.hora_gb_close(None) == capi.E_INVALID


@pytest.mark.skipif(capi.device_count() > 0, reason="needs a machine without a CUDA device")
def test_handle_run_without_a_device_is_an_error():
    from ptctcl_gb300.engine import QueryHandle
    h = QueryHandle(load_model("fischer4"), 1)
    with pytest.raises(capi.HoraError):
        h.run()
    h.close()


def test_tuner_keeps_the_default_within_the_margin():
    from ptctcl_gb300.tuner import pick
    assert pick({0: 0.99, 4: 1.0, 16: 1.01}, 4, 0.03) == 4       # 1% faster: noise
    assert pick({0: 0.90, 4: 1.0, 16: 1.01}, 4, 0.03) == 0       # 10% faster: taken
    assert pick({8: 1.2, 16: 1.0, 32: 1.1}, 16, 0.03) == 16
