"""Benchmark of the GB300 zone-graph engine: zone successors/s on the exhaustive-reachability
workload (8 automata x 10 locations, 8 clocks = 9x9 DBM, 4 binary + 1 broadcast channel, 10%
committed and 10% urgent locations, constants in [0,50], query A[] not deadlock).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--seed S]

A step is one complete query (deadlock_reachable) through the C ABI with the network in host
memory: the descriptor upload, every BFS level and the verdict readback are inside the step.
  value  = generated successors / device time of the level loop (CUDA events on the engine's
           stream, summed over the K timed steps)
  e2e    = generated successors / wall time of the C-ABI calls (host buffers in, verdict out)
The passed store of one query (hundreds of MB at this size) exceeds L2; L2 is also flushed by a
256 MB write between steps. Under torchrun each rank runs an independent replica on its own GPU
(the single-query path does not shard) and value sums successors over ranks / max time.

--impl reference times the CPU restatement of the reference's algorithm (oracle/) on the same
workload on every host core: the route it restates (deadlock_reachable's a_M route) runs in the
reference through reach_engine with the OpenMP backend (src/reachability/engine.cpp:2367,2408-2409),
so the port expands each BFS level on all host threads and inserts per key in the sequential order.
Each step is one whole query, bounded in time (a step that hits the bound reports its partial rate).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD_CONFIG = 2
WORKLOAD_SEED = int(os.environ.get("HORA_BENCH_SEED", "2483"))
# The port stops within a few hundred items of this limit (it checks its clock inside BFS levels).
CPU_SAMPLE_SECONDS = 90.0
METRIC = "zone successors/s"
UNIT = "successors/s"


def workload_name(seed: int) -> str:
    return (f"config2: 8 automata x 10 locations, 8 clocks (9x9 DBM), 4 binary + 1 broadcast channels, "
            f"A[] not deadlock, seed {seed}")


def workload(seed: int):
    from ptctcl_gb300.generator import config_instance
    return config_instance(WORKLOAD_CONFIG, seed)


def sample_clocks(stop: threading.Event, out: list):
    q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    try:
        p = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits", "-lms", "200"],
                             stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
    except OSError:
        return
    while not stop.is_set():
        line = p.stdout.readline()
        if not line:
            break
        out.append(line.strip())
    p.terminate()


def clock_summary(lines, dev_index: int):
    sm, mx, reasons = [], [], set()
    names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
    for ln in lines:
        f = [x.strip() for x in ln.split(",")]
        if len(f) < 9 or f[0] != str(dev_index):
            continue
        try:
            sm.append(float(f[1])); mx.append(float(f[2]))
        except ValueError:
            continue
        for n, v in zip(names, f[5:9]):
            if v.lower().startswith("active"):
                reasons.add(n)
    if not sm:
        return None
    return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return json.load(fh), "measured"
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def cpu_baseline(net, seconds: float, threads: int = 0):
    """The oracle port of the query on `threads` host threads (default: every core), bounded by
    `seconds`; the successors/s of the whole query, or of the levels reached when the bound hits."""
    from oracle import pyoracle
    threads = threads or os.cpu_count() or 1
    used = pyoracle.set_threads(threads)
    pyoracle.set_time_limit(seconds)
    try:
        t = time.perf_counter()
        _, st = pyoracle.deadlock_reachable(net)
        dt = time.perf_counter() - t
    finally:
        pyoracle.set_time_limit(0)
        pyoracle.set_threads(1)
    return {"value": st["generated"] / dt if dt > 0 else 0.0, "unit": UNIT, "cores": used, "kind": "port",
            "whole_query": not st["status"], "seconds": dt,
            "sample": f"{'BFS levels 1-' + str(st['levels']) + ' (the last in part)' if st['status'] else 'whole query'}"
                      f" of the workload on {used} host threads, {st['generated']} successors in {dt:.1f} s"}


def family_bytes(st, dim: int) -> dict:
    """Algorithmic bytes each kernel family of one query must move at least (int32 zones): expand
    reads every frontier zone and writes every successor; the deadlock goal reads every successor;
    the probe reads every successor, the column 0 of every stored zone it tests and the whole of
    those column 0 does not decide; the merge reads its survivors and the live zones of the keys it
    folds them into, and writes the zones it stores."""
    z, c0 = 4 * dim * dim, 4 * dim
    return {"expand": z * (st.explored + st.generated), "deadlock": z * st.generated,
            "probe": z * st.generated + c0 * st.probes + z * st.probe_full,
            "merge": z * (st.merge_surv + st.merge_live + st.nodes)}


def profiled_traffic(seed: int):
    """DRAM bytes per query of the merge kernel from the committed ncu summary of this workload
    (profiles/k_merge_dram_config2_seed<seed>.md, line `traffic_bytes_per_query: N`), or None."""
    path = os.path.join(ROOT, "profiles", f"k_merge_dram_config2_seed{seed}.md")
    try:
        for ln in open(path):
            if ln.startswith("traffic_bytes_per_query:"):
                return int(ln.split(":")[1])
    except OSError:
        pass
    return None


def roofline(st, dim: int, peaks: dict, peak_kind: str, traffic_per_query=None) -> dict:
    """HBM roofline of the dominant kernel family (CUDA-event time on the engine's stream): its
    algorithmic bytes per launch over its mean launch time, against the measured copy bandwidth;
    every family's figure beside it."""
    kern = st.kernels
    tot = sum(x["seconds"] for x in kern.values())
    fb = family_bytes(st, dim)
    per = {}
    for k, b in fb.items():
        sec, calls = kern[k]["seconds"], max(1, kern[k]["calls"])
        ach = (b / calls) / (sec / calls) / 1e9 if sec > 0 else 0.0
        per[k] = {"gbs": round(ach, 2), "bytes": int(b), "seconds": round(sec, 6), "launches": kern[k]["calls"]}
    dom = max(fb, key=lambda k: kern[k]["seconds"])
    peak = peaks.get("hbm_gbs", 1.0)
    traffic = None
    if traffic_per_query is not None and dom == "merge":
        traffic = traffic_per_query / max(1, kern[dom]["calls"])   # per launch, like bytes_per_launch
    return {"bound": "hbm", "kernel": dom, "achieved": per[dom]["gbs"], "peak": peak, "unit": "GB/s",
            "frac": per[dom]["gbs"] / peak, "traffic": traffic, "peak_source": peak_kind,
            "traffic_source": "k_merge DRAM read+write per query from the ncu capture in profiles/, per family "
                              "launch" if traffic is not None else None,
            "bytes_per_launch": per[dom]["bytes"] / max(1, kern[dom]["calls"]),
            "path_gbs": round(sum(fb.values()) / max(1e-12, st.device_seconds) / 1e9, 2),
            "families": per,
            "kernel_time_share": {k: round(v["seconds"] / max(1e-12, tot), 4) for k, v in kern.items()}}


def run_reference(args, rank, world):
    if rank != 0:
        return
    net, kind, p, q = workload(args.seed)
    vals, samples, cores, whole = [], [], 1, True
    per_step = max(5.0, min(CPU_SAMPLE_SECONDS, 240.0 / max(1, args.steps)))   # whole run within minutes
    for _ in range(args.warmup):
        cpu_baseline(net, min(2.0, per_step))
    t_all = time.perf_counter()
    for _ in range(args.steps):
        b = cpu_baseline(net, per_step)
        vals.append(b["value"]); samples.append(b["sample"])
        cores, whole = b["cores"], whole and b["whole_query"]
    dt = time.perf_counter() - t_all
    v = statistics.mean(vals) if vals else 0.0
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * dt / max(1, args.steps), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic",
            "config": {"workload": workload_name(args.seed)},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port", "whole_query": whole,
                             "sample": samples[-1] if samples else ""},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def combine_ranks(gen, dev, wall, total, dist, device):
    """Whole-job figures of N replicas: successors summed over ranks, times the max over ranks."""
    import torch
    if dist is None:
        return gen, dev, wall, total
    vals = torch.tensor([gen, dev, wall, total], dtype=torch.float64, device=device)
    g = vals.clone()
    dist.all_reduce(g, op=dist.ReduceOp.SUM)
    m = vals.clone()
    dist.all_reduce(m, op=dist.ReduceOp.MAX)
    return g[0].item(), m[1].item(), m[2].item(), m[3].item()


def percentile(xs, q):
    if not xs:
        return None
    xs = sorted(xs)
    k = min(len(xs) - 1, max(0, int(round(q / 100.0 * (len(xs) - 1)))))
    return xs[k]


def percentiles_all(finished_times, total: int, budget: float) -> dict:
    """p50/p99 time to verdict over ALL `total` instances, the unfinished ones counted as taking
    longer than the budget: a percentile that falls among them is reported as None with its flag."""
    xs = sorted(finished_times) + [float("inf")] * max(0, total - len(finished_times))
    out = {}
    for q in (50, 99):
        v = percentile(xs, q)
        out[f"p{q}_time_to_verdict_s"] = None if v is None or v == float("inf") else v
        out[f"p{q}_beyond_budget"] = v == float("inf")
    out["budget_s"] = budget
    return out


def _cpu_batch_worker(wid, nworkers, instances, budget, out, go, t_go):
    """One process of the CPU sample: once `go` is set, instances wid, wid + n, ... of config 4
    through the oracle port until t_go + budget (time.time() based; the port checks its clock
    inside levels too), one (instance, successors, finished, verdict, time) record per instance on
    `out`."""
    from oracle import pyoracle
    from ptctcl_gb300.generator import config_instance
    pyoracle.lib()
    out.put("ready")
    go.wait()
    deadline = t_go.value + budget
    for k in range(wid, instances, nworkers):
        left = deadline - time.time()
        if left <= 0:
            break
        net, kind, p, q = config_instance(4, k)
        pyoracle.set_time_limit(left)
        if kind == 0:
            v, st = pyoracle.reachable_net(net, p)
        elif kind == 1:
            v, st = pyoracle.deadlock_reachable(net)
        else:
            v, st = pyoracle.leads_to(net, p, q)
        out.put((k, st["generated"], st["status"] == 0, int(v), time.time()))
    out.put(None)


def cpu_batched_sample(instances: int, budget: float, cores: int = 0) -> dict:
    """Config 4 on the host cores: the oracle port, one instance per process at a time on every core,
    for `budget` seconds of wall time. Workers are spawned (the GPU may already be in use) and start
    together once all have loaded the port. A worker still busy a quarter of the budget after the
    deadline is stopped and its current instance is not counted."""
    import multiprocessing as mp
    import queue
    from oracle import pyoracle
    pyoracle.build()   # once, before the workers load it
    cores = cores or os.cpu_count() or 1
    ctx = mp.get_context("spawn")
    out, go, t_go = ctx.Queue(), ctx.Event(), ctx.Value("d", 0.0)
    procs = [ctx.Process(target=_cpu_batch_worker, args=(w, cores, instances, budget, out, go, t_go), daemon=True)
             for w in range(cores)]
    try:
        for pr in procs:
            pr.start()
        ready, t_start = 0, time.time()
        while ready < cores:   # every worker has imported the port before the clock starts
            try:
                if out.get(timeout=1.0) == "ready":
                    ready += 1
            except queue.Empty:
                if any(pr.exitcode is not None for pr in procs):
                    raise RuntimeError("a CPU worker exited before starting")
                if time.time() - t_start > 120:
                    raise RuntimeError("CPU workers did not start within 120 s")
        t0 = time.time()
        t_go.value = t0
        go.set()
        deadline = t0 + budget
        recs, ended = [], 0
        hard = deadline + 0.25 * budget
        while ended < cores and time.time() < hard:
            try:
                r = out.get(timeout=max(0.01, min(0.5, hard - time.time())))
            except queue.Empty:
                continue
            if r is None:
                ended += 1
            else:
                recs.append(r)
        dt = time.time() - t0
    finally:
        for pr in procs:
            if pr.is_alive():
                pr.terminate()
            pr.join(timeout=10)
    gen = sum(r[1] for r in recs)
    verdicts = {r[0]: r[3] for r in recs if r[2]}
    lat = [r[4] - t0 for r in recs if r[2]]
    return {"value": gen / dt, "unit": UNIT, "cores": cores, "kind": "port", "seconds": dt,
            "verdicts": len(verdicts), "p50_time_to_verdict_s": percentile(lat, 50),
            "p99_time_to_verdict_s": percentile(lat, 99), "stopped_workers": cores - ended,
            "sample": f"config-4 instance k on worker k mod {cores}, {budget:.0f} s",
            "_verdicts": verdicts}


def batched_compare(instances: int, budget: float, cpu_budget: float = 0.0) -> dict:
    """Config 4: `instances` seeded networks in one batched run vs the same instances one at a time
    (the plain form), each form given the same wall-time budget (some generated instances have
    millions of zones, so neither form finishes them all). Time to verdict counts from the start of
    the form's run; verdicts of instances both forms finished must agree."""
    import ctypes
    from ptctcl_gb300 import engine
    from ptctcl_gb300.generator import config_instance
    items = [config_instance(4, s) for s in range(instances)]
    batch = engine.BatchInput(items)   # descriptors built before the clock starts

    def timed(fn):
        cancel = ctypes.c_int32(0)
        tm = threading.Timer(budget, lambda: setattr(cancel, "value", 1))
        tm.start()
        t = time.perf_counter()
        out = fn(cancel)
        dt = time.perf_counter() - t
        tm.cancel()
        return out, dt

    (bv, bst), bdt = timed(lambda c: engine.batch_run(batch, cancel=c))
    b_done = [s for v, s in zip(bv, bst) if v >= 0]
    b_gen = sum(s["generated"] for s in bst)
    plain_gen, plain_done, plain_lat, t0 = 0, 0, [], time.perf_counter()
    plain_v = {}
    for k, it in enumerate(items):
        left = budget - (time.perf_counter() - t0)
        if left <= 0:
            break
        cancel = ctypes.c_int32(0)
        tm = threading.Timer(left, lambda c=cancel: setattr(c, "value", 1))
        tm.start()
        v, st = engine.batch_run([it], cancel=cancel)
        tm.cancel()
        plain_gen += st[0]["generated"]
        if v[0] >= 0:
            plain_done += 1
            plain_lat.append(time.perf_counter() - t0)
            plain_v[k] = v[0]
    pdt = time.perf_counter() - t0
    lat = [s["seconds"] for s in b_done]
    both = [k for k in plain_v if bv[k] >= 0]
    cpu = {}
    if cpu_budget > 0:
        try:
            c = cpu_batched_sample(instances, cpu_budget)
            cv = c.pop("_verdicts")
            cboth = [k for k in cv if bv[k] >= 0]
            c["verdicts_compared"] = len(cboth)
            c["verdicts_agree"] = all(cv[k] == bv[k] for k in cboth)
        except Exception as e:   # a reported baseline: its failure must not cost the GPU line
            c = {"unavailable": f"{type(e).__name__}: {e}"[:200]}
        cpu = {"cpu_port_all_cores": c}
    return {"workload": f"config4: {instances} seeded networks (clocks U[2,16], automata "
            f"U[2,10], locations U[4,12], c in [0,40], query mix 60/30/10), {budget:.0f} s budget per form",
            "batched": {"value": b_gen / bdt, "unit": UNIT, "seconds": bdt, "verdicts": len(b_done),
                        **percentiles_all(lat, instances, budget)},
            "plain_one_at_a_time": {"value": plain_gen / pdt, "unit": UNIT, "seconds": pdt, "verdicts": plain_done,
                                    **percentiles_all(plain_lat, instances, budget)},
            "speedup_successors_per_s": (b_gen / bdt) / max(1e-9, plain_gen / pdt),
            "verdicts_compared": len(both), "verdicts_agree": all(plain_v[k] == bv[k] for k in both), **cpu}


def like_for_like(config: int, seeds, cap: float, plain_budget: float) -> dict:
    """Batched vs plain on the same instances, both to completion. The plain form runs the seeded
    instances one at a time (each cancelled after `cap` seconds, the whole pass after `plain_budget`);
    the instances it finished form the set S. The batched form then runs exactly S in one call. Both
    forms did the same work, so the ratio of their successors/s is the ratio of their times; time to
    verdict is over all of S (nothing censored), and every verdict is compared."""
    import ctypes
    from ptctcl_gb300 import engine
    from ptctcl_gb300.generator import config_instance
    done_items, plain_lat, plain_v, plain_gen, plain_seeds, plain_st = [], [], [], 0, [], []
    tried, t0 = 0, time.perf_counter()
    plain_busy = 0.0
    for sd in seeds:
        if time.perf_counter() - t0 > plain_budget:
            break
        it = config_instance(config, sd)
        cancel = ctypes.c_int32(0)
        tm = threading.Timer(cap, lambda c=cancel: setattr(c, "value", 1))
        tm.start()
        t = time.perf_counter()
        v, st = engine.batch_run([it], cancel=cancel)
        dt = time.perf_counter() - t
        tm.cancel()
        tried += 1
        if v[0] >= 0 and st[0]["status"] == 0:
            done_items.append(it)
            plain_seeds.append(sd)
            plain_st.append(st[0])
            plain_v.append(v[0])
            plain_gen += st[0]["generated"]
            plain_busy += dt
            plain_lat.append(plain_busy)   # time to verdict when S alone runs one after another
    if not done_items:
        return {"instances": 0}
    batch = engine.BatchInput(done_items)
    t = time.perf_counter()
    bv, bst = engine.batch_run(batch)
    bdt = time.perf_counter() - t
    b_gen = sum(s_["generated"] for s_ in bst)
    lat = [s_["seconds"] for s_ in bst]
    return {"instances": len(done_items), "tried": tried, "per_instance_cap_s": cap,
            "plain_one_at_a_time": {"value": plain_gen / plain_busy, "unit": UNIT, "seconds": plain_busy,
                                    "p50_time_to_verdict_s": percentile(plain_lat, 50),
                                    "p99_time_to_verdict_s": percentile(plain_lat, 99)},
            "batched": {"value": b_gen / bdt, "unit": UNIT, "seconds": bdt,
                        "p50_time_to_verdict_s": percentile(lat, 50), "p99_time_to_verdict_s": percentile(lat, 99)},
            "speedup": (b_gen / bdt) / max(1e-12, plain_gen / plain_busy),
            "same_successors": b_gen == plain_gen,
            "verdicts_compared": len(bv), "verdicts_agree": list(bv) == plain_v,
            "mismatches": [{"seed": plain_seeds[k], "kind": done_items[k][1], "plain": plain_v[k], "batched": bv[k],
                            "batched_status": bst[k]["status"], "plain_generated": plain_st[k]["generated"],
                            "batched_generated": bst[k]["generated"]}
                           for k in range(len(bv)) if bv[k] != plain_v[k] or
                           bst[k]["generated"] != plain_st[k]["generated"]][:8]}


def leadsto_record(seed: int, cpu_seconds: float = 0.0) -> dict:
    """Config 3 at full size (6 automata x 8 locations, 6 clocks, p --> q): one warm-up and one timed
    query through the C ABI; the oracle port of the same query on every host core beside it."""
    from ptctcl_gb300 import engine
    from ptctcl_gb300.engine import Backend, ReachStats
    from ptctcl_gb300.generator import config_instance
    net, kind, p, q = config_instance(3, seed)
    engine.leads_to_clocks(net, p, q, Backend.Cuda, ReachStats())
    st = ReachStats()
    t = time.perf_counter()
    holds = engine.leads_to_clocks(net, p, q, Backend.Cuda, st)
    wall = time.perf_counter() - t
    rec = {"workload": f"config3 seed {seed}: 6 automata x 8 locations, 6 clocks (7x7 DBM), p --> q",
           "holds": holds, "successors": st.generated, "levels": st.levels, "graph_zones": st.stored,
           "value": st.generated / max(1e-12, st.device_seconds), "e2e": st.generated / max(1e-12, wall),
           "unit": UNIT, "time_to_verdict_s": wall,
           "decided_by": ("early witness" if (not holds and st.stored == 0) else "backward sweep" if st.stored
                           else "no reachable p-state"),
           "roofline": roofline(st, net.dim, *measured_peaks())}
    if cpu_seconds > 0:
        from oracle import pyoracle
        used = pyoracle.set_threads(os.cpu_count() or 1)
        pyoracle.set_time_limit(cpu_seconds)
        try:
            t = time.perf_counter()
            ch, cst = pyoracle.leads_to(net, p, q)
            cdt = time.perf_counter() - t
        finally:
            pyoracle.set_time_limit(0)
            pyoracle.set_threads(1)
        rec["cpu_baseline"] = {"value": cst["generated"] / cdt, "unit": UNIT, "cores": used, "kind": "port",
                               "whole_query": not cst["status"], "seconds": cdt,
                               "verdict_agrees": (ch == holds) if not cst["status"] else None}
    return rec


def run_batched(args):
    line = {"metric": METRIC, **batched_compare(args.instances, args.budget,
                                                0.0 if args.no_cpu_baseline else args.budget)}
    print(json.dumps(line), flush=True)


def serving_run(rate: float, duration: float, drain: float, budget_gb: float, inflight: int,
                serve_config: int = 3, per_request_gb: float = 0.25, max_queued: int = 64) -> dict:
    """Config 5: Poisson arrivals of requests drawn from the config-3 distribution at `rate` per
    second for `duration` seconds into the serving queue: admitted continuously while one of
    `inflight` slots is free and the `budget_gb` pool holds the request's store reservation; a request
    whose store outgrows `per_request_gb` stops with HORA_E_BUDGET (so every admitted request ends in
    bounded time), and a submission that finds `max_queued` requests waiting is rejected at once.
    Time to verdict runs from submission to result. After the arrivals the queue drains (at most
    `drain` seconds). Percentiles of time to outcome are over every accepted request (verdict or
    stopped at its limit), those of time to verdict over the requests with a verdict."""
    import ctypes
    import random
    from ptctcl_gb300 import capi
    from ptctcl_gb300.model import NetArrays, QueryArrays, Stats
    from ptctcl_gb300.generator import config_instance
    lib = capi.load()
    srv = ctypes.c_void_p()
    capi.check(lib.hora_gb_server_create(int(budget_gb * (1 << 30)), inflight, ctypes.byref(srv)), "server")
    capi.check(lib.hora_gb_server_set_limits(srv, int(per_request_gb * (1 << 30)), max_queued), "server_limits")
    rng = random.Random(5)
    # up to 2000 distinct requests, offered in turn (descriptors built before the clock)
    reqs = [config_instance(serve_config, 100000 + k) for k in range(min(2000, int(rate * duration * 1.5) + 16))]
    descs = [(NetArrays(n), QueryArrays(kd, p, q)) for n, kd, p, q in reqs]
    t0 = time.perf_counter()
    tickets, k, next_t, rejected = {}, 0, 0.0, 0
    while True:
        now = time.perf_counter() - t0
        if now >= duration:
            break
        if now >= next_t:
            na, qa = descs[k % len(descs)]
            tk = ctypes.c_int64(0)
            rc = lib.hora_gb_server_submit(srv, ctypes.addressof(na.desc), ctypes.addressof(qa.desc), ctypes.byref(tk))
            if rc == capi.OK:
                tickets[tk.value] = k % len(descs)
            elif rc == capi.E_BUDGET:
                rejected += 1
            k += 1
            next_t += rng.expovariate(rate)
        else:
            time.sleep(min(0.002, next_t - now))
    submitted = time.perf_counter() - t0
    pending, lat, out_t, gen, stopped, failed = set(tickets), [], [], 0, 0, 0
    verdict_of = {}
    t_last = submitted
    active = ctypes.c_int32(1)
    while pending and time.perf_counter() - t0 < duration + drain:
        lib.hora_gb_server_step(srv, ctypes.byref(active))
        for tk in list(pending):
            d, v, st = ctypes.c_int32(0), ctypes.c_int32(0), Stats()
            if lib.hora_gb_server_poll(srv, tk, ctypes.byref(d), ctypes.byref(v), ctypes.byref(st)) != capi.OK:
                pending.discard(tk)
                continue
            if d.value:
                pending.discard(tk)
                gen += st.generated
                t_last = time.perf_counter() - t0
                out_t.append(st.seconds)
                if st.status == capi.OK:
                    lat.append(st.seconds)
                    verdict_of[tk] = v.value
                elif st.status == capi.E_BUDGET:
                    stopped += 1
                else:
                    failed += 1
    total = time.perf_counter() - t0
    lib.hora_gb_server_destroy(srv)
    xs = sorted(out_t) + [float("inf")] * len(pending)
    o50, o99 = percentile(xs, 50), percentile(xs, 99)
    rec = {"workload": f"config{serve_config} requests, Poisson {rate:g}/s for {duration:.0f} s, "
           f"pool {budget_gb:g} GB, {inflight} in flight, {per_request_gb:g} GB per request, "
           f"at most {max_queued} waiting",
           "offered": k, "accepted": len(tickets), "rejected_at_submit": rejected,
           "verdicts": len(lat), "stopped_at_request_limit": stopped, "failed": failed,
           "unfinished": len(pending), "value": gen / max(1e-9, t_last), "unit": UNIT,
           "p50_time_to_verdict_s": percentile(lat, 50), "p99_time_to_verdict_s": percentile(lat, 99),
           "p50_time_to_outcome_s": None if o50 in (None, float("inf")) else o50,
           "p99_time_to_outcome_s": None if o99 in (None, float("inf")) else o99,
           "seconds": total, "last_result_s": t_last, "submit_seconds": submitted}
    rec["_verdicts"] = {tickets[tk]: v for tk, v in verdict_of.items()}
    return rec


def serving_plain(budget_gb: float, per_request_gb: float, seconds: float, serve_config: int = 3,
                  served=None) -> dict:
    """The plain single-instance form on the serving workload: the same request sequence run one at a
    time (one slot, the same per-request store limit) for `seconds`; its verdicts are compared with
    those the served runs gave for the same requests."""
    from ptctcl_gb300 import capi, engine
    from ptctcl_gb300.generator import config_instance
    gen, done, stopped, agree, compared = 0, 0, 0, 0, 0
    t0 = time.perf_counter()
    busy = 0.0
    k = 0
    with engine.Server(budget_bytes=int(budget_gb * (1 << 30)), max_inflight=1,
                       per_request_bytes=int(per_request_gb * (1 << 30))) as srv:
        while time.perf_counter() - t0 < seconds:
            it = config_instance(serve_config, 100000 + k)
            t = time.perf_counter()
            tk = srv.submit(*it)
            while True:
                r = srv.poll(tk)
                if r is not None:
                    break
                srv.active()
            busy += time.perf_counter() - t
            v, st = r
            gen += st["generated"]
            if st["status"] == capi.OK:
                done += 1
                for sv in served or ():
                    if k in sv:
                        compared += 1
                        agree += sv[k] == v
            else:
                stopped += 1
            k += 1
    return {"workload": f"config{serve_config} requests one at a time, {per_request_gb:g} GB per request",
            "requests": k, "verdicts": done, "stopped_at_request_limit": stopped,
            "value": gen / max(1e-9, busy), "unit": UNIT, "seconds": busy,
            "verdicts_compared_with_served": compared, "verdicts_agree": agree == compared}


def serving_sweep(rates, duration: float, drain: float, budget_gb: float, inflight: int, serve_config: int,
                  per_request_gb: float, max_queued: int, plain_seconds: float) -> dict:
    runs = [serving_run(r, duration, drain, budget_gb, inflight, serve_config, per_request_gb, max_queued)
            for r in rates]
    served = [r.pop("_verdicts") for r in runs]
    out = {"loads": runs}
    if plain_seconds > 0:
        plain = serving_plain(budget_gb, per_request_gb, plain_seconds, serve_config, served)
        out["plain_one_at_a_time"] = plain
        for r in runs:
            r["vs_plain"] = r["value"] / max(1e-12, plain["value"])
    return out


def run_serving(args):
    rates = [float(r) for r in args.rates.split(",")] if args.rates else [args.rate]
    line = {"metric": METRIC, "serving": serving_sweep(rates, args.duration, args.drain, args.budget_gb, args.inflight,
                                                       args.serve_config, args.per_request_gb, args.max_queued,
                                                       args.duration)}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--seed", type=int, default=WORKLOAD_SEED)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", default="deadlock", choices=["deadlock", "batched", "serving"])
    ap.add_argument("--instances", type=int, default=4096)
    ap.add_argument("--budget", type=float, default=60.0)
    ap.add_argument("--rate", type=float, default=100.0)
    ap.add_argument("--rates", default="", help="serving: comma-separated offered loads (req/s)")
    ap.add_argument("--leadsto-seeds", default="22,2,168",
                    help="full-size config-3 seeds recorded on the default line (empty: none)")
    ap.add_argument("--serving-seconds", type=float, default=15.0,
                    help="seconds of arrivals per load of the serving sweep added to the default line (0: leave it out)")
    ap.add_argument("--duration", type=float, default=60.0)
    ap.add_argument("--drain", type=float, default=120.0)
    ap.add_argument("--budget-gb", type=float, default=64.0)
    ap.add_argument("--inflight", type=int, default=64)
    ap.add_argument("--per-request-gb", type=float, default=0.25,
                    help="serving: a request whose store outgrows this stops with HORA_E_BUDGET")
    ap.add_argument("--max-queued", type=int, default=64,
                    help="serving: submissions that find this many requests waiting are rejected")
    ap.add_argument("--serve-config", type=int, default=3)
    ap.add_argument("--batched-budget", type=float, default=20.0,
                    help="seconds per form of the config-4 batched-vs-plain comparison added to the default "
                         "line (0: leave it out)")
    args = ap.parse_args()
    if args.workload == "batched":
        run_batched(args)
        return
    if args.workload == "serving":
        run_serving(args)
        return

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank, world)
        return

    import torch
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    from ptctcl_gb300 import capi, engine
    from ptctcl_gb300.engine import Backend, ReachStats
    capi.load()
    net, kind, p, q = workload(args.seed + rank * 0)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    verdict = None
    for _ in range(args.warmup):
        verdict = engine.deadlock_reachable(net, Backend.Cuda, ReachStats())
    stop, clk = threading.Event(), []
    th = threading.Thread(target=sample_clocks, args=(stop, clk), daemon=True)
    th.start()
    stats = []
    walls = []
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        st = ReachStats()
        tw = time.perf_counter()
        v = engine.deadlock_reachable(net, Backend.Cuda, st)
        walls.append(time.perf_counter() - tw)
        assert verdict is None or v == verdict
        verdict = v
        stats.append(st)
    barrier()
    total = time.perf_counter() - t0
    stop.set()
    gen = sum(s.generated for s in stats)
    dev = sum(s.device_seconds for s in stats)
    wall = sum(walls)
    gen_all, dev_max, wall_max, total_max = combine_ranks(gen, dev, wall, total, dist, "cuda")
    if rank != 0:
        dist.destroy_process_group()
        return
    s0 = stats[-1]
    peaks, peak_kind = measured_peaks()
    line = {
        "metric": METRIC, "value": gen_all / dev_max if dev_max > 0 else 0.0, "unit": UNIT,
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * total_max / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int32", "data": "synthetic",
        "config": {"workload": workload_name(args.seed)},
        "query": {"stored_zones": s0.stored, "successors_per_query": s0.generated, "levels": s0.levels,
                  "verdict_deadlock_reachable": bool(verdict), "l2": "flushed (256 MB write) between steps; "
                  "passed store exceeds L2", "parallelism": f"replicas x{world}"},
        "e2e": {"value": gen_all / wall_max if wall_max > 0 else 0.0, "unit": UNIT,
                "h2d_bytes_per_step": int(s0.h2d_bytes), "d2h_bytes_per_step": int(s0.d2h_bytes)},
        "gpu_launches": int(sum(s.kernel_launches for s in stats)),
    }
    line["roofline"] = roofline(s0, net.dim, peaks, peak_kind, profiled_traffic(args.seed))
    cs = clock_summary(clk, local)
    if cs:
        line["clocks"] = cs
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(net, CPU_SAMPLE_SECONDS)
    if args.batched_budget > 0 and world == 1:
        line["batched"] = batched_compare(args.instances, args.batched_budget,
                                          0.0 if args.no_cpu_baseline else args.batched_budget)
        # the same instances to completion in both forms: those the plain form finishes within 0.1 s
        # (the many small requests of the mix) and within 2 s (a few large ones bound the batch)
        line["batched_like_for_like"] = {
            f"config{c}_cap_{cap:g}s": like_for_like(c, range(base, base + args.instances), cap, args.batched_budget / 2)
            for c, base in ((4, 0), (3, 100000)) for cap in (0.1, 2.0)}
    seeds3 = [int(x) for x in args.leadsto_seeds.split(",") if x.strip()]
    if seeds3 and world == 1:
        line["config3"] = [leadsto_record(sd, 0.0 if (args.no_cpu_baseline or k) else 60.0) for k, sd in enumerate(seeds3)]
    if args.serving_seconds > 0 and world == 1:
        line["serving"] = serving_sweep((100.0, 1000.0, 5000.0), args.serving_seconds, 4 * args.serving_seconds,
                                        args.budget_gb, args.inflight, 3, args.per_request_gb, args.max_queued,
                                        args.serving_seconds)
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
