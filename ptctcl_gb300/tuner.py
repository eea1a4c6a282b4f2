"""Autotuner for the engine's per-dimension knobs (hora_gb_set_tuning), measured on the GPU at hand.

The knobs change how the level kernels are launched, never what they compute:
  long_list      the key-list length past which the passed-store probe scans a successor's key with
                 a whole warp (32 list entries per round) instead of one DBM tile (D per round);
  blocks_per_sm  the grid of the level kernels, in blocks per SM;
  group_max      the most instances of one dimension the batched form runs as one group.

For each DBM dimension D (clocks + 1) of the batched workload (config 4: clocks U[2,16], automata
U[2,10], locations U[4,12]), the tuner keeps the first `per_dim` seeded instances of that dimension
that the default configuration finishes within `cap` seconds, then times every candidate value of
each knob on exactly those instances, one knob after the other (long_list, then blocks_per_sm with
the chosen long_list, then group_max): long_list and blocks_per_sm by the summed device time of the
instances run one at a time, group_max by the wall time of one batched call over all of them; each
figure is the better of `reps` runs. A knob leaves its built-in default (long_list 4, blocks_per_sm
16, group_max 64) only for a candidate at least `margin` (3%) faster, the run-to-run spread of these
timings. Every run's verdicts and successor counts are compared with the default run's, and a
mismatch stops the tuner. The result, the measurements behind it and the device's name go to a
JSON file (`ptctcl_gb300/tuning.json` by default), which ptctcl_gb300.capi
installs whenever it loads the library.

    python -m ptctcl_gb300.tuner [--out PATH] [--per-dim 8] [--cap 0.2] [--reps 2] [--margin 0.03]
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import threading
import time

from . import capi, engine
from .generator import config_instance

LONG_LIST = (0, 4, 16, 64, 1 << 30)
BLOCKS_PER_SM = (8, 16, 32)
GROUP_MAX = (16, 32, 64)
DEFAULTS = {"long_list": 4, "blocks_per_sm": 16, "group_max": 64}


def pick(times: dict, default, margin: float):
    """The fastest candidate, or the default unless the fastest beats it by at least `margin`."""
    best = min(times, key=lambda x: times[x])
    return best if times[best] < times[default] * (1.0 - margin) else default


def _run_one(item, cap: float):
    """One instance through the batched entry point, cancelled after `cap` seconds: (verdict, stats)."""
    cancel = ctypes.c_int32(0)
    tm = threading.Timer(cap, lambda: setattr(cancel, "value", 1))
    tm.start()
    try:
        v, st = engine.batch_run([item], cancel=cancel)
    finally:
        tm.cancel()
    return v[0], st[0]


def _table(dim: int, **knobs) -> dict:
    return {k: {dim: v} for k, v in knobs.items() if v is not None}


def select(dim_items: dict, per_dim: int, cap: float) -> dict:
    """Per dimension, the instances the default configuration finishes within `cap` seconds, with
    their default verdicts and successor counts."""
    capi.set_tuning({})
    out = {}
    for d, items in sorted(dim_items.items()):
        keep = []
        for it in items:
            v, st = _run_one(it, cap)
            if v >= 0 and st["status"] == capi.OK:
                keep.append((it, v, st["generated"]))
            if len(keep) >= per_dim:
                break
        if keep:
            out[d] = keep
    return out


def _single_pass(keep, table: dict, reps: int) -> float:
    """Summed device seconds of the instances run one at a time under `table` (the best of `reps`)."""
    capi.set_tuning(table)
    best = None
    for _ in range(reps):
        tot = 0.0
        for it, v0, g0 in keep:
            v, st = engine.batch_run([it])
            if v[0] != v0 or st[0]["generated"] != g0:
                raise RuntimeError(f"tuning changed a result: verdict {v[0]} vs {v0}, successors "
                                   f"{st[0]['generated']} vs {g0}")
            tot += st[0]["device_seconds"]
        best = tot if best is None else min(best, tot)
    return best


def _batch_pass(keep, table: dict, reps: int) -> float:
    """Wall seconds of one batched call over all the instances under `table` (the best of `reps`)."""
    capi.set_tuning(table)
    items = [it for it, _, _ in keep]
    best = None
    for _ in range(reps):
        t = time.perf_counter()
        v, st = engine.batch_run(items)
        dt = time.perf_counter() - t
        for k, (it, v0, g0) in enumerate(keep):
            if v[k] != v0 or st[k]["generated"] != g0:
                raise RuntimeError("tuning changed a result in the batched form")
        best = dt if best is None else min(best, dt)
    return best


def tune(seeds: int = 1200, per_dim: int = 8, cap: float = 0.2, reps: int = 2, margin: float = 0.03) -> dict:
    dim_items = {}
    for s in range(seeds):
        it = config_instance(4, s)
        dim_items.setdefault(it[0].dim, [])
        if len(dim_items[it[0].dim]) < 4 * per_dim:
            dim_items[it[0].dim].append(it)
    chosen = select(dim_items, per_dim, cap)
    choice = {"long_list": {}, "blocks_per_sm": {}, "group_max": {}}
    measured = {}
    for d, keep in chosen.items():
        m = {"instances": len(keep), "successors": sum(g for _, _, g in keep)}
        t_ll = {x: _single_pass(keep, _table(d, long_list=x), reps) for x in LONG_LIST}
        ll = pick(t_ll, DEFAULTS["long_list"], margin)
        t_bp = {x: _single_pass(keep, _table(d, long_list=ll, blocks_per_sm=x), reps) for x in BLOCKS_PER_SM}
        bp = pick(t_bp, DEFAULTS["blocks_per_sm"], margin)
        t_gm = {x: _batch_pass(keep, _table(d, long_list=ll, blocks_per_sm=bp, group_max=x), reps) for x in GROUP_MAX}
        gm = pick(t_gm, DEFAULTS["group_max"], margin)
        choice["long_list"][d], choice["blocks_per_sm"][d], choice["group_max"][d] = ll, bp, gm
        m.update({"long_list_device_s": {str(k): v for k, v in t_ll.items()},
                  "blocks_per_sm_device_s": {str(k): v for k, v in t_bp.items()},
                  "group_max_wall_s": {str(k): v for k, v in t_gm.items()}})
        measured[d] = m
    capi.set_tuning({})
    return {"choice": choice, "measured": measured, "device": _device_name(),
            "when": time.strftime("%Y-%m-%dT%H:%M:%SZ", time.gmtime()),
            "workload": f"config-4 instances that finish within {cap} s, up to {per_dim} per dimension",
            "margin": margin}


def _device_name() -> str:
    try:
        import torch
        return torch.cuda.get_device_name(0)
    except Exception:   # the name is informative only
        return "unknown"


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=capi.TUNING_PATH)
    ap.add_argument("--seeds", type=int, default=1200)
    ap.add_argument("--per-dim", type=int, default=8)
    ap.add_argument("--cap", type=float, default=0.2)
    ap.add_argument("--reps", type=int, default=2)
    ap.add_argument("--margin", type=float, default=0.03)
    a = ap.parse_args()
    os.environ["HORA_GB_TUNING"] = "0"   # measure from the built-in defaults
    res = tune(a.seeds, a.per_dim, a.cap, a.reps, a.margin)
    with open(a.out, "w") as f:
        json.dump(res, f, indent=1, sort_keys=True)
    print(json.dumps(res["choice"]))


if __name__ == "__main__":
    main()
