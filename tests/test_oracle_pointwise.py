"""The oracle's DBM algebra checked point by point on one to three clocks (test infrastructure: it
pins the restatement beyond the reference's own known answers). With integer constants, every
region of n clocks holds a point whose coordinates are multiples of 1/(n+1), so a quarter grid over
[0, 8] decides emptiness, inclusion and the exact convex union (the merge the passed store relies
on, netengine_metal.mm:310-335) for zones bounded by 7."""
import numpy as np
import pytest

from oracle.pyoracle import Dbm

INF = 1 << 30
NEG_INF = -(1 << 29)   # the a_LU "-inf" bound


def raw(v, weak):
    return (v << 1) | (1 if weak else 0)


def grid(nclk, hi=8.0, step=0.25):
    ax = np.arange(0.0, hi + 1e-9, step)
    g = np.stack(np.meshgrid(*([ax] * nclk), indexing="ij"), -1).reshape(-1, nclk)
    return np.concatenate([np.zeros((g.shape[0], 1)), g], 1)   # column 0 is the reference clock


def member(d, P):
    ok = np.ones(P.shape[0], bool)
    for i in range(d.shape[0]):
        for j in range(d.shape[0]):
            b = int(d[i, j])
            if i == j or b >= INF:
                continue
            diff = P[:, i] - P[:, j]
            ok &= (diff <= (b >> 1)) if (b & 1) else (diff < (b >> 1))
    return ok


def random_zone(rng, nclk):
    """A canonical zone: the positive orthant, 1-4 random difference constraints, every clock <= 7
    (None when the constraints are contradictory)."""
    z = Dbm(nclk)
    for k in range(1, nclk + 1):
        z.free(k)
    for _ in range(int(rng.integers(1, 5))):
        i, j = (int(x) for x in rng.choice(nclk + 1, 2, replace=False))
        if not z.constrain(i, j, raw(int(rng.integers(-6, 7)), bool(rng.integers(0, 2)))):
            return None
    for k in range(1, nclk + 1):
        if not z.constrain(k, 0, raw(7, True)):
            return None
    return None if z.empty() else z


@pytest.mark.parametrize("nclk", [1, 2, 3])
def test_zones_are_their_points(nclk):
    """Non-empty zones hold grid points; constrain intersects the point set with a half-space;
    includes is inclusion of point sets."""
    rng = np.random.default_rng(11 + nclk)
    P = grid(nclk)
    zones = [z for z in (random_zone(rng, nclk) for _ in range(400)) if z is not None]
    assert len(zones) > 100
    for z in zones:
        assert member(z.d, P).any()
    for z in zones[:150]:
        i, j = (int(x) for x in rng.choice(nclk + 1, 2, replace=False))
        b = raw(int(rng.integers(-7, 8)), bool(rng.integers(0, 2)))
        c = z.copy()
        nonempty = c.constrain(i, j, b)
        diff = P[:, i] - P[:, j]
        half = (diff <= (b >> 1)) if (b & 1) else (diff < (b >> 1))
        want = member(z.d, P) & half
        assert nonempty == bool(want.any())
        if nonempty:
            assert np.array_equal(member(c.d, P), want)
    for a, b in zip(zones[:200:2], zones[1:200:2]):
        ma, mb = member(a.d, P), member(b.d, P)
        assert a.includes(b) == bool(np.all(ma | ~mb))
        assert b.includes(a) == bool(np.all(mb | ~ma))


@pytest.mark.parametrize("nclk", [1, 2, 3])
def test_try_union_is_exactly_convexity(nclk):
    """try_union succeeds iff the entrywise-max hull adds no point outside a and b, and then holds
    exactly the points of a and b."""
    rng = np.random.default_rng(29 + nclk)
    P = grid(nclk)
    merged = refused = 0
    for _ in range(600):
        a, b = random_zone(rng, nclk), random_zone(rng, nclk)
        if a is None or b is None:
            continue
        ma, mb = member(a.d, P), member(b.d, P)
        hull = np.maximum(a.d, b.d)
        convex = bool(np.all(~member(hull, P) | ma | mb))
        u = a.copy()
        assert u.try_union(b) == convex
        if convex:
            merged += 1
            assert np.array_equal(u.d, hull)
            assert np.array_equal(member(u.d, P), ma | mb)
        else:
            refused += 1
            assert np.array_equal(u.d, a.d)   # a failed union leaves a unchanged
    assert merged > 20 and refused > 20


@pytest.mark.parametrize("nclk", [1, 2, 3])
def test_delay_reset_extrapolate_and_simulation_laws(nclk):
    """delay and Extra_LU+ only add points; reset puts the clock at 0; a_LU simulation is reflexive,
    implied by inclusion, and transitive along chains of inclusions."""
    rng = np.random.default_rng(47 + nclk)
    P = grid(nclk, hi=12.0, step=0.25)
    zones = [z for z in (random_zone(rng, nclk) for _ in range(300)) if z is not None]
    for z in zones[:120]:
        mz = member(z.d, P)
        up = z.copy().delay()
        assert up.includes(z) and np.all(member(up.d, P) | ~mz)
        assert np.array_equal(up.copy().delay().d, up.d)
        k = int(rng.integers(1, nclk + 1))
        r = z.copy().reset(k)
        mr = member(r.d, P)
        assert mr.any() and np.all(P[mr, k] == 0)
        bounds = np.array([NEG_INF, 0, 1, 2, 3, 4, 5], np.int64)   # NEG_INF: the clock has no bound
        L = np.concatenate([[0], rng.choice(bounds, nclk)]).astype(np.int32)
        U = np.concatenate([[0], rng.choice(bounds, nclk)]).astype(np.int32)
        e = z.copy().extrapolate_lu_plus(L, U)
        assert e.includes(z)
        assert z.alu_le(z, L, U)
    for a, b in zip(zones[:200:2], zones[1:200:2]):
        L = np.concatenate([[0], rng.integers(0, 8, nclk)]).astype(np.int32)
        U = np.concatenate([[0], rng.integers(0, 8, nclk)]).astype(np.int32)
        if b.includes(a):
            assert a.alu_le(b, L, U)
        # a chain a' ⊆ a and a ≼ b gives a' ≼ b
        if a.alu_le(b, L, U):
            sub = a.copy()
            i, j = (int(x) for x in rng.choice(nclk + 1, 2, replace=False))
            if sub.constrain(i, j, raw(int(rng.integers(-3, 4)), True)):
                assert sub.alu_le(b, L, U)
