"""ctypes binding of libhora_gb300.so (the C ABI of include/hora_gb300.h)."""
from __future__ import annotations

import ctypes
import os

import numpy as np

from .model import P32, Stats, NetDesc, PredDesc, QueryDesc

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libhora_gb300.so")

OK, E_INVALID, E_NOT_SUPPORTED, E_CUDA, E_OVERFLOW, E_TIMEOUT, E_BUDGET, E_NOMEM, E_CANCELLED, E_NO_DEVICE = range(10)
BACKEND_SEQ, BACKEND_OMP, BACKEND_CUDA, BACKEND_METAL = range(4)

EXPORTS = (
    "hora_gb_last_error", "hora_gb_abi_version", "hora_gb_device_count", "hora_gb_reachable_net",
    "hora_gb_deadlock_reachable", "hora_gb_leads_to", "hora_gb_exists_invariant",
    "hora_gb_exists_invariant_trace", "hora_gb_expand",
    "hora_gb_has_deadlock",
    "hora_gb_batch_run", "hora_gb_server_create", "hora_gb_server_submit", "hora_gb_server_step",
    "hora_gb_server_poll", "hora_gb_server_destroy", "hora_gb_server_set_limits", "hora_gb_set_tuning", "hora_gb_has_deadlock_noalloc",
    "hora_gb_open", "hora_gb_run", "hora_gb_trace", "hora_gb_close",
)

_lib = None


class HoraError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"hora_gb status {code}: {msg}")
        self.code = code


def load(build_if_missing: bool = True):
    """Load the in-tree library. Raises if it is missing and cannot be built: there is no fallback."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        if not build_if_missing:
            raise ImportError(f"{LIB_PATH} is missing; run ptctcl_gb300.build.build()")
        from . import build
        build.build()
    L = ctypes.CDLL(LIB_PATH)
    I32, I64, U64 = ctypes.c_int32, ctypes.c_int64, ctypes.c_uint64
    VP = ctypes.c_void_p
    L.hora_gb_last_error.restype = ctypes.c_char_p
    L.hora_gb_abi_version.restype = I32
    L.hora_gb_device_count.argtypes = [ctypes.POINTER(I32)]
    L.hora_gb_device_count.restype = I32
    L.hora_gb_reachable_net.argtypes = [VP, VP, I32, VP, ctypes.POINTER(I32)]
    L.hora_gb_reachable_net.restype = I32
    L.hora_gb_deadlock_reachable.argtypes = [VP, I32, VP, VP, ctypes.POINTER(I32)]
    L.hora_gb_deadlock_reachable.restype = I32
    L.hora_gb_leads_to.argtypes = [VP, VP, VP, I32, VP, ctypes.POINTER(I32)]
    L.hora_gb_leads_to.restype = I32
    L.hora_gb_exists_invariant.argtypes = [VP, VP, I32, VP, ctypes.POINTER(I32)]
    L.hora_gb_exists_invariant.restype = I32
    L.hora_gb_exists_invariant_trace.argtypes = [VP, VP, I32, VP, ctypes.POINTER(I32), I32, ctypes.POINTER(I32),
                                                 P32, P32, P32, P32, ctypes.POINTER(I32), ctypes.POINTER(I32)]
    L.hora_gb_exists_invariant_trace.restype = I32
    L.hora_gb_expand.argtypes = [VP, I32, P32, P32, P32, P32, P32, ctypes.POINTER(ctypes.c_uint8), I32, I64,
                                 P32, P32, P32, P32, P32, ctypes.POINTER(I64)]
    L.hora_gb_expand.restype = I32
    L.hora_gb_has_deadlock.argtypes = [VP, I32, P32, P32, P32, P32]
    L.hora_gb_has_deadlock.restype = I32
    L.hora_gb_has_deadlock_noalloc.argtypes = [VP, I32, VP, VP, VP, VP]
    L.hora_gb_has_deadlock_noalloc.restype = I32
    L.hora_gb_open.argtypes = [VP, VP, ctypes.POINTER(VP)]
    L.hora_gb_open.restype = I32
    L.hora_gb_run.argtypes = [VP, ctypes.POINTER(I32), VP]
    L.hora_gb_run.restype = I32
    L.hora_gb_trace.argtypes = [VP, I32, ctypes.POINTER(I32), P32, P32, P32, P32, ctypes.POINTER(I32),
                                ctypes.POINTER(I32)]
    L.hora_gb_trace.restype = I32
    L.hora_gb_close.argtypes = [VP]
    L.hora_gb_close.restype = I32
    L.hora_gb_batch_run.argtypes = [I32, VP, VP, P32, VP, VP]
    L.hora_gb_batch_run.restype = I32
    L.hora_gb_server_create.argtypes = [U64, I32, ctypes.POINTER(VP)]
    L.hora_gb_server_create.restype = I32
    L.hora_gb_server_submit.argtypes = [VP, VP, VP, ctypes.POINTER(I64)]
    L.hora_gb_server_submit.restype = I32
    L.hora_gb_server_set_limits.argtypes = [VP, U64, I32]
    L.hora_gb_server_set_limits.restype = I32
    L.hora_gb_server_step.argtypes = [VP, ctypes.POINTER(I32)]
    L.hora_gb_server_step.restype = I32
    L.hora_gb_server_poll.argtypes = [VP, I64, ctypes.POINTER(I32), ctypes.POINTER(I32), VP]
    L.hora_gb_server_poll.restype = I32
    L.hora_gb_server_destroy.argtypes = [VP]
    L.hora_gb_server_destroy.restype = I32
    L.hora_gb_set_tuning.argtypes = [P32, P32, P32, I32]
    L.hora_gb_set_tuning.restype = I32
    _lib = L
    apply_tuning()
    return L


TUNING_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tuning.json")


def set_tuning(table: dict):
    """Install a per-dimension tuning table (hora_gb_set_tuning): {"long_list": {D: n}, "group_max":
    {D: n}, "blocks_per_sm": {D: n}}, D the DBM dimension; missing entries keep the defaults."""
    n = 18
    arrs = []
    for key in ("long_list", "group_max", "blocks_per_sm"):
        a = np.full(n, -1, np.int32)
        for d, v in (table.get(key) or {}).items():
            if 0 <= int(d) < n:
                a[int(d)] = int(v)
        arrs.append(a)
    check(load().hora_gb_set_tuning(p32(arrs[0]), p32(arrs[1]), p32(arrs[2]), n), "set_tuning")


def apply_tuning(path: str = TUNING_PATH):
    """The tuner's measured table, when one is installed beside the library (ptctcl_gb300/tuning.json);
    without one, or with HORA_GB_TUNING=0, the built-in defaults."""
    if os.environ.get("HORA_GB_TUNING", "1") == "0" or not os.path.exists(path):
        set_tuning({})
        return
    import json
    import warnings
    try:
        with open(path) as f:
            table = json.load(f).get("choice", {})
        set_tuning(table)
    except (OSError, ValueError, AttributeError, TypeError) as e:   # a damaged table: the defaults
        warnings.warn(f"ignoring {path}: {e}")
        set_tuning({})


def last_error() -> str:
    return load().hora_gb_last_error().decode(errors="replace")


def check(rc: int, what: str = ""):
    if rc != OK:
        raise HoraError(rc, f"{what}: {last_error()}")


def device_count() -> int:
    n = ctypes.c_int32(0)
    load().hora_gb_device_count(ctypes.byref(n))
    return n.value


def p32(a: np.ndarray):
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(P32)
