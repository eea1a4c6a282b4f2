"""The allocation-free deadlock entry point, for callers that cannot allocate device memory.

hora_gb_has_deadlock_noalloc takes device buffers the caller already owns and keeps the compiled
network in the library's static device array; it must give exactly the answers of the allocating
entry point hora_gb_has_deadlock (integer results: exact equality), on two calls in a row (the
array keeps the previous call's contents), and must refuse a network too large for the array.
Kept in the file collected last, so that a failure here comes after every other test has run.
"""
import ctypes

import numpy as np
import pytest

from ptctcl_gb300 import capi, engine
from ptctcl_gb300.generator import config_instance
from oracle import pyoracle
from ptctcl_gb300.model import NetArrays, Network, Process, Location, Edge, c_le, c_ge
from states import sample_states

pytestmark = pytest.mark.gpu


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.int32)).cuda()


@pytest.mark.parametrize("cfg,seed", [(2, 23), (1, 3), (4, 0)])
def test_noalloc_matches_allocating_entry_point(cfg, seed):
    torch = pytest.importorskip("torch")
    lib = capi.load()
    net = config_instance(cfg, seed)[0]
    smp = sample_states(net, nmax=150, depth=5)
    assert smp is not None
    locs, ints, zones, _, _ = smp
    n = locs.shape[0]
    want = engine.has_deadlock(net, locs, ints, zones)        # the allocating entry point
    np.testing.assert_array_equal(want, pyoracle.has_deadlock(net, locs, ints, zones))   # and the oracle
    na = NetArrays(net)
    d_locs, d_zones = _dev(torch, locs), _dev(torch, zones)
    d_ints = _dev(torch, ints) if len(net.ints) else None
    d_out = torch.full((n,), -7, dtype=torch.int32, device="cuda")
    for _ in range(2):                                        # two calls in a row share the array
        d_out.fill_(-7)
        torch.cuda.synchronize()
        rc = lib.hora_gb_has_deadlock_noalloc(ctypes.addressof(na.desc), n, d_locs.data_ptr(),
                                              d_ints.data_ptr() if d_ints is not None else None,
                                              d_zones.data_ptr(), d_out.data_ptr())
        assert rc == capi.OK, capi.last_error()
        assert capi.last_error() == ""                       # a successful call leaves no message
        got = d_out.cpu().numpy()
        np.testing.assert_array_equal(got.astype(bool), want)
        assert set(np.unique(got)) <= {0, 1}


def test_noalloc_rejects_a_network_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    lib = capi.load()
    # one process with 30000 guarded edges: its tables need far more than the 1 MiB array
    edges = [Edge(0, 0, guard=[c_ge(1, k % 7), c_le(1, 9)], resets=[1]) for k in range(30000)]
    big = Network(1, [Process("P", [Location("A", [c_le(1, 9)])], edges, 0)])
    na = NetArrays(big)
    d = torch.zeros(4, dtype=torch.int32, device="cuda")
    rc = lib.hora_gb_has_deadlock_noalloc(ctypes.addressof(na.desc), 1, d.data_ptr(), None, d.data_ptr(),
                                          d.data_ptr())
    assert rc == capi.E_INVALID
    assert "static scratch" in capi.last_error()
