"""Reachable symbolic states sampled with the oracle, as inputs for the per-state parity tests."""
import numpy as np

from oracle import pyoracle
from ptctcl_gb300.model import Network


def sample_states(net: Network, nmax: int = 200, depth: int = 6, qmask=None, seed: int = 0):
    """BFS from the initial state through the oracle's successor function (no subsumption); up to
    nmax distinct (locs, ints, zone) triples, in discovery order."""
    ok, l0, i0, z0 = pyoracle.initial_state(net, qmask)
    if not ok:
        return None
    L, U, _, _, _ = pyoracle.static_bounds(net)
    seen = set()
    out_l, out_i, out_z = [], [], []

    def add(l, i, z):
        k = (l.tobytes(), i.tobytes(), z.tobytes())
        if k in seen:
            return False
        seen.add(k)
        out_l.append(l.copy()); out_i.append(i.copy()); out_z.append(z.copy())
        return True

    add(l0, i0, z0)
    frontier = [(l0, i0, z0)]
    for _ in range(depth):
        if not frontier or len(out_l) >= nmax:
            break
        fl = np.stack([f[0] for f in frontier]); fi = np.stack([f[1] for f in frontier]) if len(net.ints) else np.zeros((len(frontier), 0), np.int32)
        fz = np.stack([f[2] for f in frontier])
        r = pyoracle.expand(net, fl, fi, fz, L, U, qmask)
        nxt = []
        for k in range(len(r["src"])):
            if add(r["locs"][k], r["ints"][k], r["zones"][k]):
                nxt.append((r["locs"][k], r["ints"][k], r["zones"][k]))
                if len(out_l) >= nmax:
                    break
        frontier = nxt
    ni = len(net.ints)
    return (np.stack(out_l), np.stack(out_i) if ni else np.zeros((len(out_l), 0), np.int32), np.stack(out_z), L, U)
