"""Pin the oracle's DBM algebra against the reference's known answers (tests/dbm_tests.cpp)."""
import numpy as np

from oracle.pyoracle import Dbm, fed_covers
from ptctcl_gb300.model import le, lt, INF


def zone1(lo, hi):
    """1-clock zone [lo, hi] built the way dbm_tests.cpp:14-21 builds it (hi < 0: unbounded)."""
    z = Dbm(1)
    z.delay()
    if hi >= 0:
        z.constrain(1, 0, le(hi))
    z.constrain(0, 1, le(-lo))
    z.close()
    return z


def test_basic():                                   # dbm_tests.cpp:24-36
    z = zone1(0, 5)
    assert not z.empty()
    assert z.get(1, 0) == le(5)
    assert z.get(0, 1) == le(0)
    e = Dbm(1)
    e.delay()
    e.constrain(1, 0, le(5))
    assert not e.constrain(0, 1, le(-6))
    assert e.empty()


def test_reset_delay():                             # dbm_tests.cpp:38-45
    z = zone1(2, 5)
    z.reset(1)
    assert z.get(1, 0) == le(0) and z.get(0, 1) == le(0)
    z.delay()
    assert z.get(1, 0) == INF
    assert z.get(0, 1) == le(0)


def test_inclusion():                               # dbm_tests.cpp:47-52
    a, b = zone1(0, 5), zone1(3, 5)
    assert a.includes(b)
    assert not b.includes(a)
    assert a.includes(a)


def test_extrapolate():                             # dbm_tests.cpp:54-60 (Extra_LU+ with L = U = M)
    z = zone1(0, 5)
    z.extrapolate_lu_plus([0, 4], [0, 4])
    assert z.get(1, 0) == INF
    assert z.get(0, 1) == le(0)


def test_two_clocks_diagonal():                     # dbm_tests.cpp:62-75
    z = Dbm(2)
    z.delay()
    assert z.constrain(1, 0, le(5))
    assert z.constrain(0, 2, le(-2))
    assert z.constrain(1, 2, le(1))
    assert not z.empty()
    w = z.copy()
    assert not w.constrain(2, 1, le(-5)) and w.empty()


def test_selftest():                                # app/main.cpp:26-41: [0,5] includes [3,5]
    assert zone1(0, 5).includes(zone1(3, 5))


def test_fed_covers_matches_pointwise():
    """Federation covering against explicit enumeration over a 1-clock grid."""
    rng = np.random.default_rng(7)
    for _ in range(300):
        lo = int(rng.integers(0, 8)); hi = lo + int(rng.integers(0, 8))
        z = zone1(lo, hi)
        ws = []
        for _k in range(int(rng.integers(0, 4))):
            a = int(rng.integers(0, 10)); b = a + int(rng.integers(0, 6))
            ws.append(zone1(a, b))
        # half-integer grid points decide coverage of closed integer intervals
        pts = [x / 2 for x in range(2 * lo, 2 * hi + 1)]
        want = all(any(w_lo <= p <= w_hi for (w_lo, w_hi) in
                       [(-(w.get(0, 1) >> 1), w.get(1, 0) >> 1) for w in ws]) for p in pts)
        assert fed_covers(z, ws) == want


def test_try_union_exact():
    """Convex union of 1-clock intervals: convex iff they touch or overlap."""
    for (a0, a1, b0, b1) in [(0, 3, 3, 5), (0, 3, 4, 5), (0, 3, 1, 2), (2, 4, 0, 1), (2, 4, 0, 2)]:
        a, b = zone1(a0, a1), zone1(b0, b1)
        convex = not (a1 < b0 or b1 < a0)
        assert a.try_union(b) == convex
        if convex:
            assert a.get(1, 0) == le(max(a1, b1)) and a.get(0, 1) == le(-min(a0, b0))


def test_alu_le_reflexive_and_inclusion():
    L = np.array([0, 5, 5], np.int32); U = np.array([0, 5, 5], np.int32)
    z = Dbm(2); z.delay(); z.constrain(1, 0, le(3)); z.constrain(0, 2, lt(-1))
    big = Dbm(2); big.delay()
    assert z.alu_le(z, L, U)
    assert z.alu_le(big, L, U)
    assert not big.alu_le(z, L, U)
