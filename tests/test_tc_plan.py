"""Bounds of the tensor-core kernel's launch plans, checked on the CPU.

tests/cpp/tc_plan_check.cc plans random decimation groups (1-4 classes of up
rates 1-4, 2-64 taps, 1-32 channels, D 2-400, row-split limits 1-8) with the
library's own planner (libfalcon_dsp_gb300/csrc/fdsp_tc_plan.h: row split,
merge sets, pair windows, launches) and checks every shared-memory read the
kernel derives from a plan against the plan's sizes: the A operand's records
of each MMA, the taps of each work set inside its merged window, the staged
span of the bulk copy, and the shared-memory budget of the chosen buffer
count.  No GPU is involved.
"""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "tc_plan_check.cc")
CUDA_INC = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")


def test_tc_launch_plans_stay_in_bounds(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not available")
    if not os.path.exists(os.path.join(CUDA_INC, "cuda_runtime.h")):
        pytest.skip("CUDA headers not available")
    exe = str(tmp_path / "tc_plan_check")
    cmd = [cxx, "-std=c++17", "-O2", "-Wall", "-Werror", "-I", os.path.join(ROOT, "libfalcon_dsp_gb300", "csrc"),
           "-I", os.path.join(ROOT, "include"), "-I", CUDA_INC, SRC, "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe, "20000"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    ok, cases, launches, mmas = r.stdout.split()
    assert ok == "ok" and int(cases) == 20000 and int(launches) > 20000 and int(mmas) > 100000
