"""Generate tests/golden/full_size_counts.json: the oracle's verdict and counts for whole queries
at the benchmark's full sizes -- config 2 (8 automata x 10 locations, 8 clocks, A[] not deadlock)
and config 3 (6 automata x 8 locations, 6 clocks, p --> q) -- so the GPU suite can compare them
without re-running the oracle (minutes per query even on every host core).

Usage:  python tests/golden/make_full_size.py
"""
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import pyoracle  # noqa: E402
from ptctcl_gb300.generator import config_instance  # noqa: E402

SEEDS = (1055, 2483)   # 0.31M and 1.45M stored zones
# config 3: violated by the early witness after 12 BFS levels (10.7M successors), and after 21 levels
# (110M successors); holding after the whole reachability pass (2.97M successors, no p-state
# reachable, so the subsumed graph is empty)
LEADSTO_SEEDS = (22, 2, 168)
KEYS = ("explored", "generated", "expanded", "stored", "keys", "levels")


def main():
    pyoracle.set_threads(os.cpu_count() or 1)
    rows = []
    for seed in LEADSTO_SEEDS:
        net, kind, p, q = config_instance(3, seed)
        t = time.perf_counter()
        holds, st = pyoracle.leads_to(net, p, q)
        dt = time.perf_counter() - t
        assert st["status"] == 0, st
        rows.append({"config": 3, "seed": seed, "holds": bool(holds), **{k: int(st[k]) for k in KEYS}})
        print(f"config 3 seed {seed}: {rows[-1]} ({dt:.0f} s)", flush=True)
    for seed in SEEDS:
        net, kind, p, q = config_instance(2, seed)
        t = time.perf_counter()
        verdict, st = pyoracle.deadlock_reachable(net)
        dt = time.perf_counter() - t
        assert st["status"] == 0, st
        rows.append({"config": 2, "seed": seed, "deadlock_reachable": bool(verdict),
                     **{k: int(st[k]) for k in KEYS}})
        print(f"config 2 seed {seed}: {rows[-1]} ({dt:.0f} s)", flush=True)
    with open(os.path.join(HERE, "full_size_counts.json"), "w") as fh:
        json.dump(rows, fh, indent=1)
        fh.write("\n")


if __name__ == "__main__":
    main()
