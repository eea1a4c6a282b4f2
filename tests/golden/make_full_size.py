"""Generate tests/golden/full_size_counts.json: the oracle's verdict and counts for the
deadlock workloads the bench runs at full size (config 2: 8 automata x 10 locations, 8 clocks,
A[] not deadlock), so the GPU suite can compare whole queries at those sizes without re-running
the single-threaded oracle (several minutes per query).

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
KEYS = ("explored", "generated", "expanded", "stored", "keys", "levels")


def main():
    rows = []
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
