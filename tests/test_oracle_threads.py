"""The oracle's multi-core port of the reachability route (the CPU baseline's all-core sample) gives
the sequential loop's verdicts and counts: each key's insertions keep the sequential order."""
import pytest

from oracle import pyoracle
from ptctcl_gb300.generator import config_instance

KEYS = ("explored", "generated", "stored", "keys", "levels", "probes")


@pytest.mark.parametrize("cfg,seed", [(1, 3), (1, 5), (2, 3), (2, 10), (2, 23), (4, 2), (4, 5)])
def test_threads_match_sequential(cfg, seed):
    net, kind, p, q = config_instance(cfg, seed)
    run = (lambda: pyoracle.reachable_net(net, p)) if kind == 0 else (lambda: pyoracle.deadlock_reachable(net))
    try:
        pyoracle.set_threads(1)
        want, wst = run()
        if pyoracle.set_threads(4) == 1:
            pytest.skip("oracle built without OpenMP")
        got, gst = run()
    finally:
        pyoracle.set_threads(1)
    assert got == want
    for k in KEYS:
        assert gst[k] == wst[k], (k, gst[k], wst[k])


@pytest.mark.parametrize("seed", [6, 20])
def test_threads_match_sequential_leadsto(seed):
    """Phase 1 of p --> q runs the same multi-core level; verdict and counts are unchanged."""
    net, kind, p, q = config_instance(3, seed)
    try:
        pyoracle.set_threads(1)
        want, wst = pyoracle.leads_to(net, p, q)
        if pyoracle.set_threads(4) == 1:
            pytest.skip("oracle built without OpenMP")
        got, gst = pyoracle.leads_to(net, p, q)
    finally:
        pyoracle.set_threads(1)
    assert got == want
    for k in ("explored", "generated", "stored", "keys", "levels"):
        assert gst[k] == wst[k], (k, gst[k], wst[k])
