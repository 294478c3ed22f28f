"""The march's jump over a run of skipped samples equals the sample-by-sample
loop it replaces.

The kernels step t by the rounded sequence t, t+dt, ... (integrateBrick,
deviceCode.cpp:271-296).  Inside a binade [2^e, 2^(e+1)) every float is a
multiple of 2^(e-23); when dt is too, each t + dt is exact until t crosses
the next power of two, so a run of samples in an empty macrocell is taken as
jumps t = fmaf(j, dt, t) to the binade's end, the crossing step as the loop
takes it, and so on to the macrocell's exit.  tests/cpp/exact_steps_check.cpp
compiles the very header the kernels use (aloha_gb300/csrc/steps.h) for the
host and compares jump and loop, bit for bit, on random bricks; the GPU
parity tests then pin whole frames and sample counts to the oracle, which
keeps the loop.
"""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_jump_equals_loop(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not found")
    exe = str(tmp_path / "exact_steps_check")
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I", os.path.join(ROOT, "aloha_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "cpp", "exact_steps_check.cpp"), "-o", exe], check=True)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stdout + out.stderr
    fields = out.stdout.split()
    stats = dict(zip(fields[0::2], (int(v) for v in fields[1::2])))
    assert stats["mismatches"] == 0
    assert stats["jumped"] > 10**6 and stats["exact"] > stats["bricks"] // 4 and stats["crossings"] > 1000
