"""The host loops' persistent worker pool (forestfv_public_gb300/csrc/ffv_internal.h):
exact coverage of large loops, nested loops, concurrent callers and a forked child, compiled
for the host and run as a program (a deadlock fails through the timeout)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "c", "pool_check.cpp")
OUT = os.path.join(ROOT, "tests", "c", "_build")


def test_pool_loops_nested_concurrent_and_forked():
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    os.makedirs(OUT, exist_ok=True)
    exe = os.path.join(OUT, "pool_check")
    subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-Werror", "-pthread",
                    "-I" + os.path.join(ROOT, "forestfv_public_gb300", "csrc"), SRC, "-o", exe],
                   check=True, capture_output=True, text=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert " 0 failures" in r.stdout
