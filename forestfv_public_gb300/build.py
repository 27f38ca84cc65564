"""In-tree build of the CUDA/C++ library (forestfv_public_gb300/_lib/libffv.so).

Every translation unit is compiled for sm_103a only, in parallel, then linked into one
shared library whose exported symbols are the C ABI of include/ffv.h.  The FP64 kernels
are compiled with --fmad=false so that they round every multiply and add separately, as
the reference's C code does.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
LIBDIR = os.path.join(PKG, "_lib")
LIB = os.path.join(LIBDIR, "libffv.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
          "-I" + os.path.join(ROOT, "include")]

# per-file extra flags
SOURCES = {
    "ffv_mesh.cpp": ["-Xcompiler", "-ffp-contract=off"],
    "ffv_tags.cpp": [],
    "ffv_io.cpp": [],
    "ffv_regrid.cpp": [],
    "ffv_api.cu": [],
    "ffv_m0_fp64.cu": ["--fmad=false"],
    "ffv_m5_fp64.cu": ["--fmad=false"],
    "ffv_m5_fp32.cu": [],
    "ffv_noalloc.cu": [],
    "ffv_mlp.cu": [],
    "ffv_m0_tags.cu": [],
    "ffv_adapt.cu": [],
}


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build forestfv_public_gb300")


def _compile(src: str, extra: list[str], objdir: str, verbose: bool) -> str:
    obj = os.path.join(objdir, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc(), *ARCH, *COMMON, *extra, "-c", os.path.join(CSRC, src), "-o", obj]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose and r.stderr:
        sys.stderr.write(r.stderr)
    return obj


def build(verbose: bool = False) -> str:
    os.makedirs(LIBDIR, exist_ok=True)
    objdir = os.path.join(LIBDIR, "obj")
    os.makedirs(objdir, exist_ok=True)
    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda kv: _compile(kv[0], kv[1], objdir, verbose), SOURCES.items()))
    tmp = LIB + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


def build_oracle() -> str:
    """CPU restatement the tests check the CUDA path against (oracle/_build/libffv_oracle.so)."""
    odir = os.path.join(ROOT, "oracle")
    out = os.path.join(odir, "_build")
    os.makedirs(out, exist_ok=True)
    lib = os.path.join(out, "libffv_oracle.so")
    srcs = sorted(os.path.join(odir, f) for f in os.listdir(odir) if f.endswith(".c"))
    cmd = ["gcc", "-std=c99", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
           "-o", lib, *srcs, "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed: {' '.join(cmd)}\n{r.stderr}")
    return lib


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
    print(build_oracle())
