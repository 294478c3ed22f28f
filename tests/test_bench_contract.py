"""bench.py's reference arm on the CPU: one JSON line with the contract's keys.

`bench.py --impl reference` times the reference path on the host cores: the
reference's own raygen compiled on the CPU (oracle/_ref) where its sources or
build are present, else the CPU restatement (the oracle), on the same metric,
unit and config as the GPU arm; under several ranks only rank 0 prints.  Run
here at a small volume and image so that it takes a few seconds.
"""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ARGS = ["--impl", "reference", "--n", "64", "--size", "64", "--cameras", "4", "--steps", "3", "--warmup", "3"]


def _run(env_extra=None, extra=()):
    env = dict(os.environ)
    env.update(env_extra or {})
    return subprocess.run([sys.executable, os.path.join(ROOT, "bench.py")] + ARGS + list(extra), capture_output=True,
                          text=True, timeout=600, env=env, cwd=ROOT)


def _line(out):
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1
    return json.loads(lines[0])


def test_reference_arm_prints_the_contract_line():
    d = _line(_run())
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
                "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["impl"] == "reference"
    assert d["unit"] == "Gsamples/s" and d["value"] > 0 and d["higher_is_better"] is True
    assert d["steps"] == 3 and d["warmup"] == 3 and d["n_gpus"] == 1
    assert d["config"]["volume"] == [64, 64, 64] and d["config"]["image"] == [64, 64]
    assert "64^3" in d["config"]["workload"]
    # the same config object as the GPU arm's, so the two lines compare as one workload
    sys.path.insert(0, ROOT)
    import bench
    args = type("A", (), {"n": 64, "size": 64})()
    assert d["config"] == bench.workload_config(args, 4, 1)
    cb = d["cpu_baseline"]
    from oracle import reference as R
    assert cb["kind"] == ("reference" if R.loadable() else "port")
    assert cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["unit"] == d["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_reference_arm_kinds_time_the_same_samples():
    """The reference's own build and the restatement march the same bands:
    their sample counts (value x time) agree to the pinned tolerance."""
    sys.path.insert(0, ROOT)
    from oracle import reference as R
    if not R.available():
        pytest.skip("the reference sources are not present")
    port = _line(_run(extra=["--reference-kind", "port"]))
    ref = _line(_run(extra=["--reference-kind", "reference"]))
    assert port["cpu_baseline"]["kind"] == "port" and ref["cpu_baseline"]["kind"] == "reference"
    samples = [d["value"] * 1e9 * d["ms_per_step"] * 1e-3 * d["steps"] for d in (port, ref)]
    assert abs(samples[0] - samples[1]) <= 1e-3 * samples[0]


def test_reference_arm_other_ranks_print_nothing():
    out = _run({"RANK": "1", "WORLD_SIZE": "2"})
    assert out.returncode == 0, out.stderr[-2000:]
    assert out.stdout.strip() == ""


@pytest.mark.gpu
def test_gpu_arm_prints_the_contract_line():
    """The GPU arm at a small size: value, e2e with the copied bytes, the
    roofline of the dominant kernel, the CPU baseline, clocks and the count of
    this library's kernel launches."""
    pytest.importorskip("torch")
    import torch
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    args = ["--n", "128", "--size", "256", "--cameras", "8", "--steps", "4", "--warmup", "3", "--no-adjoint",
            "--no-large", "--no-batched", "--cpu-seconds", "1"]
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py")] + args, capture_output=True, text=True,
                         timeout=900, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    d = json.loads([ln for ln in out.stdout.splitlines() if ln.strip()][-1])
    assert d["unit"] == "Gsamples/s" and d["value"] > 0 and d["steps"] == 4 and d["warmup"] == 3
    assert d["gpu_launches"] >= d["steps"]
    e2e = d["e2e"]
    assert e2e["value"] > 0 and e2e["h2d_bytes_per_step"] > 0 and e2e["d2h_bytes_per_step"] == 256 * 256 * 4
    r = d["roofline"]
    assert r["bound"] == "hbm" and r["unit"] == "GB/s" and r["achieved"] > 0 and r["peak"] > 0
    assert abs(r["frac"] - r["achieved"] / r["peak"]) < 1e-9
    cb = d["cpu_baseline"]
    assert cb["value"] > 0 and cb["cores"] >= 1 and cb["kind"] == "port"
    clk = d["clocks"]
    assert {"sm_mhz", "sm_max_mhz", "samples", "reasons"} <= set(clk)
    assert not {"hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown"} & set(clk["reasons"])

