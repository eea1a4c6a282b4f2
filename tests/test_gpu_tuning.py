"""The tuning table (hora_gb_set_tuning) changes how the level kernels are launched, never what they
compute: with the probe's warp-wide scan for every list or for none, a small or large grid, and
batched groups of 1 or 64 instances, every verdict and every count equals the default run's."""
import pytest

from ptctcl_gb300 import capi, engine
from ptctcl_gb300.generator import config_instance
from test_gpu_parity import C4_SMALL, small_config3

pytestmark = pytest.mark.gpu

COUNTS = ("explored", "generated", "stored", "keys", "levels")


def _items():
    items = [config_instance(2, 23), config_instance(1, 3)] + [config_instance(4, s) for s in C4_SMALL[:8]]
    items += [small_config3(s) for s in (1, 17, 23)]
    return items


def _dims(items):
    return sorted({it[0].dim for it in items})


@pytest.mark.parametrize("knobs", [
    {"long_list": 0, "blocks_per_sm": 8, "group_max": 1},
    {"long_list": 1 << 30, "blocks_per_sm": 32, "group_max": 64},
    {"long_list": 16, "blocks_per_sm": 4, "group_max": 3},
], ids=["warp-every-list", "tile-every-list", "mixed"])
def test_tuning_changes_no_result(knobs):
    items = _items()
    capi.set_tuning({})
    ref = [engine.batch_run([it]) for it in items]
    refb = engine.batch_run(items)
    try:
        capi.set_tuning({k: {d: v for d in _dims(items)} for k, v in knobs.items()})
        got = [engine.batch_run([it]) for it in items]
        gotb = engine.batch_run(items)
    finally:
        capi.apply_tuning()
    for k, ((rv, rs), (gv, gs)) in enumerate(zip(ref, got)):
        assert gv[0] == rv[0], k
        for c in COUNTS:
            assert gs[0][c] == rs[0][c], (k, c)
    assert gotb[0] == refb[0]
    for k in range(len(items)):
        for c in COUNTS:
            assert gotb[1][k][c] == refb[1][k][c], (k, c)
