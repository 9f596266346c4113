"""bench.py keeps its JSON contract: one line with the metric, the timing keys, the end-to-end
number, the roofline of the dominant kernel, the CPU baseline and the launch count.

Runs bench.py itself (on a reduced 64-qubit case and a small batch) on the GPU.
"""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

KEYS = ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
        "vs_baseline", "dtype", "data", "config", "e2e", "roofline", "cpu_baseline", "gpu_launches", "clocks")


def bench_line(*args):
    r = subprocess.run([sys.executable, "bench.py", *args], cwd=ROOT, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout[-3000:]
    return json.loads(lines[0])


@pytest.mark.gpu
def test_single_state_line():
    d = bench_line("--steps", "3", "--warmup", "3", "--k", "14", "--gates", "300", "--cpu-seconds", "1")
    for k in KEYS:
        assert k in d, k
    assert d["metric"] == "amp-updates/s" and d["unit"] == "amp-updates/s"
    assert d["value"] > 0 and d["n_gpus"] == 1 and d["steps"] == 3 and d["warmup"] == 3
    assert d["higher_is_better"] is True and d["scaling"] == "weak" and d["dtype"] == "f64"
    assert "workload" in d["config"]
    e = d["e2e"]
    assert e["value"] > 0 and e["unit"] == d["unit"]
    assert e["h2d_bytes_per_step"] > 0 and e["d2h_bytes_per_step"] > 0
    rf = d["roofline"]
    assert rf["bound"] == "hbm" and rf["unit"] == "GB/s"
    assert rf["achieved"] > 0 and rf["peak"] > 0
    assert abs(rf["frac"] - rf["achieved"] / rf["peak"]) < 1e-12
    cb = d["cpu_baseline"]
    assert cb["value"] > 0 and cb["kind"] == "port" and cb["cores"] >= 1 and cb["sample"]
    assert cb["single_thread"]["value"] > 0 and cb["single_thread"]["cores"] == 1 and cb["cpu"]
    assert d["gpu_launches"] > 0
    assert d["config"]["workload"].startswith("c3") and d["config"]["qubits"] == 64
    du = d["device_amp_updates"]
    assert 0 < du["per_step"] <= du["all_gates_per_step"] and du["value"] <= d["value"]
    assert rf["fp64_pipe"]["peak_fma_lane_ops_per_s"] > 1e11
    f32 = d["fp32"]
    assert f32["value"] > 0 and f32["dtype"] == "f32" and f32["fidelity_vs_fp64"] >= 1 - 1e-6


@pytest.mark.gpu
def test_batch_line():
    d = bench_line("--workload", "c4", "--circuits", "16", "--steps", "3", "--warmup", "3", "--no-cpu-baseline",
                   "--precision", "32")
    for k in KEYS:
        assert k in d, k
    assert d["value"] > 0 and d["dtype"] == "f32" and d["gpu_launches"] > 0
    assert d["e2e"]["value"] > 0 and d["e2e"]["d2h_bytes_per_step"] > 0
    assert d["fidelity_vs_fp64"]["min_fidelity"] >= 1 - 1e-6
