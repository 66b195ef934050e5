"""The host thread pool the plan build splits its phases over (spearfish_gb300/csrc/
sf_hostpool.h), on the CPU: a small C++ driver (tests/hostpool_check.cpp) checks that every
index is visited once, chunks are contiguous and deterministic, and concurrent callers all
finish with the right sums."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_host_pool(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "hostpool_check")
    src = os.path.join(ROOT, "tests", "hostpool_check.cpp")
    inc = os.path.join(ROOT, "spearfish_gb300", "csrc")
    r = subprocess.run([cxx, "-std=c++17", "-O2", "-pthread", "-I", inc, src, "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("OK"), r.stdout
