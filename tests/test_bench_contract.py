"""bench.py's JSON line.  The reference arm on the CPU (it needs no GPU): rank 0 prints one
line with the keys of the bench contract, its e2e copies nothing, and any other rank exits
0 without work.  The headline arm on the GPU: roofline, e2e with the bytes it copies, the
launch count and the clock record."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CMD = [sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "2", "--warmup", "1"]


def _run(env_extra):
    env = dict(os.environ, **env_extra)
    return subprocess.run(CMD, capture_output=True, text=True, timeout=900, cwd=ROOT, env=env)


def test_reference_arm_prints_one_contract_line():
    r = _run({})
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["impl"] == "reference"
    assert d["value"] > 0 and d["steps"] == 2 and d["warmup"] == 1 and d["higher_is_better"] is True
    assert "workload" in d["config"]
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["unit"] == d["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
    # the reference's own kernels on the GPU are timed beside it where a GPU is present
    rg = d["reference_gpu"]
    assert rg is None or ("unavailable" in rg) or rg["dda_cluster_bitset"]["ms"] > 0


def test_reference_arm_other_ranks_exit_quietly():
    r = _run({"RANK": "1", "LOCAL_RANK": "1", "WORLD_SIZE": "2"})
    assert r.returncode == 0, r.stderr[-2000:]
    assert not [ln for ln in r.stdout.splitlines() if ln.startswith("{")]


@pytest.mark.gpu
def test_headline_arm_prints_one_contract_line():
    """The headline arm on the GPU: roofline, cpu_baseline (skipped here), clocks, e2e with
    the copied bytes and the launch count."""
    cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--steps", "3", "--warmup", "3", "--no-cpu-baseline",
           "--serving-jobs", "6"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=900, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["value"] > 0 and d["n_gpus"] == 1 and d["steps"] == 3 and d["warmup"] >= 3
    assert d["config"]["fallback_prims"] == 0
    roof = d["roofline"]
    assert roof["bound"] == "hbm" and roof["unit"] == "GB/s" and 0 < roof["frac"] == roof["achieved"] / roof["peak"]
    e2e = d["e2e"]
    assert e2e["value"] > 0 and e2e["h2d_bytes_per_step"] > 0 and e2e["d2h_bytes_per_step"] == 1024 * 1024 * 64 * 4
    assert d["gpu_launches"] == 6 * 3
    assert d["clocks"] is None or set(d["clocks"]) >= {"sm_mhz", "sm_max_mhz", "reasons"}  # None: no nvidia-smi
    # the forms, measured after the headline's timed region
    b = d["batched"]
    assert b["value"] > 0 and b["plain_per_cluster_calls"] > 0 and b["clusters"] == 256
    assert b["batched_over_plain"] == b["value"] / b["plain_per_cluster_calls"]
    sv = d["serving"]
    assert sv["jobs"] == 6 and sv["jobs_per_s"] > 0 and sv["latency_p99_s"] >= sv["latency_p50_s"] > 0
    assert sv["serial_plain"]["jobs_per_s"] > 0
