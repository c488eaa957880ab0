"""bench.py's reference arm (the reference's algorithm on the host cores) and its JSON line, on CPU:
workload 1, one step.  The GPU arm's line is checked where a GPU runs it."""
from __future__ import annotations

import json
import os
import subprocess
import sys
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
CMD = [sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--config", "1",
       "--steps", "2", "--warmup", "1"]


def _run(env_extra=None):
    env = dict(os.environ, **(env_extra or {}))
    t0 = time.perf_counter()
    r = subprocess.run(CMD, capture_output=True, text=True, timeout=600, env=env, cwd=ROOT)
    r.wall_s = time.perf_counter() - t0
    return r


def test_reference_arm_prints_one_contract_line():
    r = _run()
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
                "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config", "impl",
                "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["impl"] == "reference" and d["steps"] == 2 and d["higher_is_better"] is False
    assert d["value"] > 0 and d["value"] == d["ms_per_step"]
    assert d["config"]["workload"].startswith("ALS config 1:")
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["value"] == d["value"] and cb["cores"] >= 1 and cb["sample"]
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["unit"] == d["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
    # whole epochs, really run: the steps' claimed time fits inside the process's own wall time
    assert d["steps"] * d["ms_per_step"] / 1e3 <= r.wall_s
    assert "whole epochs" in cb["sample"]


def test_reference_arm_does_not_load_the_product_library():
    """The CPU reference arm generates its workload with the oracle-side build of the generator:
    the product's libals_gb300.so is never mapped into its process."""
    probe = ("import runpy, sys; sys.argv = %r; "
             "runpy.run_path(%r, run_name='__main__'); "
             "maps = open('/proc/self/maps').read(); "
             "assert 'libals_gb300' not in maps, 'product library loaded'; print('CLEAN')"
             % (["bench.py"] + CMD[2:], str(ROOT / "bench.py")))
    r = subprocess.run([sys.executable, "-c", probe], capture_output=True, text=True,
                       timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    assert "CLEAN" in r.stdout


def test_reference_arm_runs_on_rank_zero_only():
    r = _run({"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1"})
    assert r.returncode == 0, r.stderr[-2000:]
    assert not [ln for ln in r.stdout.splitlines() if ln.startswith("{")]


def test_roofline_traffic_comes_from_the_committed_capture():
    """The GPU arm's roofline.traffic is read from profiles/dram_traffic.txt for the default
    workload and plan; other workloads report null rather than a borrowed figure."""
    import argparse

    sys.path.insert(0, str(ROOT))
    import bench

    a = argparse.Namespace(config=3, scale=1.0, solve="auto")
    u, v = bench.load_traffic(a, "U", "bf16"), bench.load_traffic(a, "V", "bf16")
    assert u is not None and v is not None
    # the U half's DRAM bytes stay near its algorithmic floor (8 B per rating + 800 B per row)
    floor = 8 * 98_600_426 + 800 * 480_189
    assert 0.9 * floor < u < 1.3 * floor
    assert bench.load_traffic(argparse.Namespace(config=2, scale=1.0, solve="auto"), "U",
                              "bf16") is None
