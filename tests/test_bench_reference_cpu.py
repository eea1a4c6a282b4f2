"""The reference arm of the bench (the oracle port timed on host cores) prints one JSON line with
the same metric, unit and workload as the GPU arm; it needs no GPU."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_contract_line():
    out = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "0"],
                         cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, out.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["metric"] == "zone successors/s" and d["unit"] == "successors/s"
    assert d["higher_is_better"] is True and d["n_gpus"] == 1 and d["steps"] == 1
    assert d["value"] > 0
    assert d["config"] == {"workload": d["config"]["workload"]} and d["config"]["workload"].startswith("config2")
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert "BFS levels 1-" in cb["sample"] or "whole query" in cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_cpu_batched_sample_is_bounded_and_counts_verdicts():
    """The all-core CPU sample of the batched workload (the oracle port on spawned workers) ends
    close to its budget and reports the instances it finished."""
    import time
    sys.path.insert(0, ROOT)
    import bench
    t = time.time()
    r = bench.cpu_batched_sample(64, 3.0, cores=2)
    assert time.time() - t < 3.0 * 1.25 + 60   # worker start-up (imports) is outside the budget
    assert r["cores"] == 2 and r["kind"] == "port" and r["unit"] == "successors/s"
    assert 3.0 <= r["seconds"] <= 3.0 * 1.25 + 1
    assert r["value"] > 0 and r["verdicts"] == len(r["_verdicts"]) >= 1
    assert all(v in (0, 1) for v in r["_verdicts"].values())


def test_roofline_from_family_counters():
    """The roofline names the family with the most kernel time and divides its own algorithmic
    bytes by its own time; every family is reported beside it."""
    sys.path.insert(0, ROOT)
    import bench
    from types import SimpleNamespace
    st = SimpleNamespace(explored=10, generated=100, probes=50, probe_full=5, merge_surv=40, merge_live=60, nodes=30,
                         device_seconds=1.0,
                         kernels={"expand": {"seconds": 0.1, "calls": 2}, "probe": {"seconds": 0.2, "calls": 2},
                                  "deadlock": {"seconds": 0.05, "calls": 2}, "group": {"seconds": 0.01, "calls": 4},
                                  "merge": {"seconds": 0.4, "calls": 2}, "other": {"seconds": 0.01, "calls": 3}})
    r = bench.roofline(st, 9, {"hbm_gbs": 1000.0}, "measured")
    z = 4 * 81
    assert r["kernel"] == "merge"
    assert r["families"]["merge"]["bytes"] == z * (40 + 60 + 30)
    assert r["families"]["probe"]["bytes"] == z * 100 + 36 * 50 + z * 5
    assert abs(r["achieved"] - z * 130 / 0.4 / 1e9) < 0.01
    assert abs(r["frac"] - r["achieved"] / 1000.0) < 1e-12
