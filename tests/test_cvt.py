"""The integer-pipe FP64 <-> FP32 conversions of the FP32-flux form
(forestfv_public_gb300/csrc/ffv_cvt.cuh), compiled for the host, against the compiler's
conversions: bit-identical on random patterns, ties, range edges and special values."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "c", "cvt_check.cpp")
OUT = os.path.join(ROOT, "tests", "c", "_build")


def test_conversions_match_hardware_rounding():
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    os.makedirs(OUT, exist_ok=True)
    exe = os.path.join(OUT, "cvt_check")
    subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-Werror",
                    "-I" + os.path.join(ROOT, "forestfv_public_gb300", "csrc"), SRC, "-o", exe],
                   check=True, capture_output=True, text=True)
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "0 mismatches" in r.stdout
