"""Generate tests/golden/full_size_counts.json: the oracle's verdict and counts for whole queries
at the benchmark's full sizes -- config 2 (8 automata x 10 locations, 8 clocks, A[] not deadlock)
and config 3 (6 automata x 8 locations, 6 clocks, p --> q) -- so the GPU suite can compare them
without re-running the oracle (minutes per query even on every host core); and config 5: the first
requests of the serving workload's sequence (config-3 instances, seeds 100000 + k) that the oracle
decides within a time limit, for the served-against-oracle test.

Usage:  python tests/golden/make_full_size.py [--serving-only]
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
SERVING_REQUESTS = 16       # requests 100000 .. 100015 of the serving sequence are tried
SERVING_LIMIT_S = 40.0      # the oracle's time limit per request; requests past it are left out


def serving_rows():
    rows = []
    pyoracle.set_time_limit(SERVING_LIMIT_S)
    try:
        for k in range(SERVING_REQUESTS):
            seed = 100000 + k
            net, kind, p, q = config_instance(3, seed)
            t = time.perf_counter()
            holds, st = pyoracle.leads_to(net, p, q)
            dt = time.perf_counter() - t
            if st["status"] != 0:
                print(f"config 5 request {seed}: past {SERVING_LIMIT_S:.0f} s, left out", flush=True)
                continue
            rows.append({"config": 5, "seed": seed, "holds": bool(holds), **{k_: int(st[k_]) for k_ in KEYS}})
            print(f"config 5 request {seed}: {rows[-1]} ({dt:.0f} s)", flush=True)
    finally:
        pyoracle.set_time_limit(0)
    return rows


def main():
    pyoracle.set_threads(os.cpu_count() or 1)
    path = os.path.join(HERE, "full_size_counts.json")
    if "--serving-only" in sys.argv:
        with open(path) as fh:
            rows = [r for r in json.load(fh) if r["config"] != 5]
        rows += serving_rows()
        with open(path, "w") as fh:
            json.dump(rows, fh, indent=1)
            fh.write("\n")
        return
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
    rows += serving_rows()
    with open(path, "w") as fh:
        json.dump(rows, fh, indent=1)
        fh.write("\n")


if __name__ == "__main__":
    main()
