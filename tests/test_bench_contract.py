"""The benchmark's JSON line (no GPU): the reference arm on the CPU-runnable
configuration prints one line with every key of the contract, and the
workload list holds the configurations and the rows' workloads."""
import json
import os
import subprocess
import sys

import pytest

from conftest import ROOT


def _run(args, timeout=300):
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py")] + args, cwd=ROOT,
                         capture_output=True, text=True, timeout=timeout)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, out.stdout[-2000:]
    return json.loads(lines[0])


def test_reference_arm_line(oracle):
    d = _run(["--impl", "reference", "--workload", "config1", "--steps", "1", "--warmup", "1"])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
              "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
              "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference"
    assert d["value"] > 0 and d["steps"] == 1 and d["warmup"] == 1
    # one gradient evaluation split over the ranks: total work fixed
    assert d["higher_is_better"] is True and d["scaling"] == "strong"
    # the same config object as the GPU arm's line (bench._config)
    for k in ("workload", "solves_per_step", "grid", "periods", "receivers", "mode", "l2",
              "parallelism"):
        assert k in d["config"], k
    assert "-O3" in d["cpu_baseline"]["build"]
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] in ("port", "reference") and cb["cores"] >= 1
    assert cb["sample"]
    e = d["e2e"]
    assert e["value"] == d["value"] and e["unit"] == d["unit"]
    assert e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0


def test_workload_choices():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--help"], cwd=ROOT,
                         capture_output=True, text=True, timeout=120)
    assert out.returncode == 0
    for w in ("config1", "config2", "config4", "serving", "dropin", "smooth", "kernel3d",
              "worklist", "topo"):
        assert w in out.stdout, w


@pytest.mark.gpu
def test_our_arm_line():
    d = _run(["--workload", "config1", "--steps", "3", "--warmup", "3", "--no-cpu-baseline"],
             timeout=900)
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
              "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config", "e2e",
              "gpu_launches", "roofline", "clocks"):
        assert k in d, k
    assert d["value"] > 0 and d["n_gpus"] == 1 and d["gpu_launches"] > 0
    r = d["roofline"]
    for k in ("bound", "achieved", "peak", "unit", "frac"):
        assert k in r, k
    assert 0 < r["frac"] < 2
    e = d["e2e"]
    assert e["value"] > 0 and e["h2d_bytes_per_step"] > 0 and e["d2h_bytes_per_step"] > 0
    c = d["clocks"]
    assert "sm_mhz" in c and "reasons" in c
