"""The library's host visibility orders (aloha_gb300/csrc/order.cpp) on the
CPU: tests/cpp/order_check.cpp compiles the library's own order.cpp and checks,
on random uneven brick grids, eye points and rank assignments, that every pair
of bricks is listed in an order some separating plane justifies (the eye on
the first one's side, or in the gap), that each rank's bricks follow the brick
order, and that the eye-independent split trees cached per brick set give the
same schedules as freshly built ones.  The GPU parity tests check the same
orders against the oracle through whole frames.
"""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_visibility_orders(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not found")
    exe = str(tmp_path / "order_check")
    csrc = os.path.join(ROOT, "aloha_gb300", "csrc")
    subprocess.run([cxx, "-O2", "-std=c++17", "-I", csrc, "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "order_check.cpp"), os.path.join(csrc, "order.cpp"), "-o", exe],
                   check=True)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stdout + out.stderr
    fields = out.stdout.split()
    stats = dict(zip(fields[0::2], (int(v) for v in fields[1::2])))
    assert stats["violations"] == 0 and stats["cases"] > 10000
