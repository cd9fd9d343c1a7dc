"""Bounds and coverage of the tensor-core planner, checked on the CPU.

tests/cpp/tc_plan_check.cc plans random channel sets (1-6 decimation groups
of 1-3 classes, up rates 1-4, 1-70 taps per phase, D 1-400, and every 17th
case a long single-channel FIR of 200-5000 taps) with the library's own
planner (libfalcon_dsp_gb300/csrc/fdsp_tc_plan.h) and checks what the
kernels derive from each plan: TMA coordinates and tensor-map rows inside the
split buffer, each output's window inside [history | block] and inside its
merge set's chunked window, B images, stages and tensor-memory columns inside
their budgets, per-CTA item ranges partitioning every merge set, and every
output of every channel written exactly once.  No GPU is involved.
"""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "tc_plan_check.cc")


def test_tc_plans_stay_in_bounds_and_cover_every_output(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not available")
    exe = str(tmp_path / "tc_plan_check")
    cmd = [cxx, "-std=c++17", "-O2", "-Wall", "-Werror", "-I", os.path.join(ROOT, "libfalcon_dsp_gb300", "csrc"),
           SRC, "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe, "2000"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    ok, cases, msets, items = r.stdout.split()
    assert ok == "ok" and int(cases) == 2000 and int(msets) > 5000 and int(items) > 100000
