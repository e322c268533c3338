"""bench.py's JSON line on the GPU: one line on stdout with every key of the
benchmark contract (metric, value, e2e with its copied bytes, roofline with
its traffic, cpu_baseline, clocks, gpu_launches), on a short run without the
PCG blocks."""
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.timeout(900)
def test_bench_line_has_the_contract_keys():
    cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--steps", "3", "--warmup", "3", "--no-pcg",
           "--cpu-seconds", "0.5"]
    p = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=850)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [ln for ln in p.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, p.stdout[-2000:]
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "e2e", "gpu_launches", "roofline",
              "cpu_baseline", "clocks"):
        assert k in d, k
    assert d["n_gpus"] == 1 and d["steps"] == 3 and d["warmup"] == 3 and d["value"] > 0
    assert d["unit"] == "GDOF/s" and d["dtype"] == "f64" and d["higher_is_better"] is True
    assert "workload" in d["config"]
    e2e = d["e2e"]
    assert e2e["value"] > 0 and e2e["h2d_bytes_per_step"] > 0 and e2e["d2h_bytes_per_step"] > 0
    assert e2e["bit_identical_to_device_result"] is True
    r = d["roofline"]
    for k in ("bound", "achieved", "peak", "unit", "frac", "traffic"):
        assert k in r, k
    assert r["bound"] == "fp64" and r["achieved"] > 0 and r["peak"] > 0
    assert abs(r["frac"] - r["achieved"] / r["peak"]) < 1e-9
    cb = d["cpu_baseline"]
    assert cb["value"] > 0 and cb["cores"] >= 1 and cb["kind"] == "port" and cb["sample"]
    assert d["gpu_launches"] >= d["steps"]
    assert "sm_mhz" in d["clocks"] and "reasons" in d["clocks"]
