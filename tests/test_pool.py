"""The stream server's device pool bookkeeping (RangePool in
libfalcon_dsp_gb300/csrc/fdsp_pool.h), checked on the CPU by
tests/cpp/pool_check.cc against a byte map over random alloc/release
sequences: aligned pieces inside the range that never overlap, refusals only
when no free run fits, exact free-byte accounting and full coalescing once
everything is released.  No GPU is involved."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "pool_check.cc")


def test_range_pool_against_a_byte_map(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not available")
    exe = str(tmp_path / "pool_check")
    cmd = [cxx, "-std=c++17", "-O2", "-Wall", "-Werror", "-I", os.path.join(ROOT, "libfalcon_dsp_gb300", "csrc"),
           SRC, "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe, "60"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    ok, rounds, allocs, failed = r.stdout.split()
    assert ok == "ok" and int(rounds) == 60 and int(allocs) > 60000 and int(failed) > 0
