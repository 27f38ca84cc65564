"""The boundary called from C: tests/c/bridge.c includes include/ffv.h, links the library and
runs the reference-side bridge sequence (leaves -> ffv_mesh_build -> ffv_create ->
ffv_set_mesh -> per step upload, ffv_step, download) on a fixture the reference made; the
final state must carry the reference's bits."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, load_golden

from forestfv_public_gb300 import leaves_from_paths

SRC = os.path.join(ROOT, "tests", "c", "bridge.c")
OUT = os.path.join(ROOT, "tests", "c", "_build")


def compile_bridge(built_lib, link: bool = True) -> str:
    os.makedirs(OUT, exist_ok=True)
    exe = os.path.join(OUT, "bridge")
    libdir = os.path.dirname(built_lib)
    cmd = ["gcc", "-std=c99", "-O2", "-Wall", "-Werror", "-I" + os.path.join(ROOT, "include"), SRC]
    if link:
        cmd += ["-L" + libdir, "-lffv", "-Wl,-rpath," + libdir,
                "-Wl,-rpath,/usr/local/cuda/lib64", "-o", exe]
    else:
        cmd += ["-c", "-o", exe + ".o"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def test_bridge_compiles_against_the_header(built_lib):
    """C99 with -Wall -Werror against include/ffv.h, linked against the library."""
    compile_bridge(built_lib)


@pytest.mark.gpu
def test_bridge_sequence_gives_the_reference_bits(built_lib, tmp_path):
    exe = compile_bridge(built_lib)
    g = load_golden("m0_sphere_amr")
    lv = leaves_from_paths(tuple(g["ntrees"]), g["root"], g["level"],
                           g["adrs"][:, 2:].astype(np.int64))
    n = lv.n
    head = np.array(list(g["ntrees"]) + list(g["bc_sides"]) +
                    [int(g["steps"]), int(g["order"]), int(g["rk_steps"])], np.int32)
    case = tmp_path / "case.bin"
    with open(case, "wb") as f:
        f.write(head.tobytes())
        f.write(np.int64(n).tobytes())
        f.write(np.array([1.0 / max(g["ntrees"]), float(g["dt"]), float(g["gamma"]),
                          float(g["pinf"])]).tobytes())
        f.write(np.ascontiguousarray(lv.tree_ijk, np.int32).tobytes())
        f.write(np.ascontiguousarray(lv.level, np.int32).tobytes())
        f.write(np.ascontiguousarray(lv.cell_ijk, np.int32).tobytes())
        f.write(np.ascontiguousarray(g["S_init"], np.float64).tobytes())
    out = tmp_path / "out.bin"
    r = subprocess.run([exe, str(case), str(out)], capture_output=True, text=True)
    assert r.returncode == 0, (r.returncode, r.stdout, r.stderr)
    S = np.fromfile(out, np.float64).reshape(n, 5)
    assert np.array_equal(S, g["S_final"])
