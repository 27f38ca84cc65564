"""The C-ABI library loads and exports every function include/ffv.h declares."""
import ctypes
import os
import re

from conftest import ROOT


def declared():
    src = open(os.path.join(ROOT, "include", "ffv.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(ffv_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_the_path():
    names = declared()
    for must in ("ffv_create", "ffv_set_mesh", "ffv_upload_state", "ffv_stage", "ffv_step",
                 "ffv_download_state", "ffv_cfl_dt", "ffv_destroy", "ffv_mesh_build"):
        assert must in names


def test_library_exports_every_declared_symbol(built_lib):
    lib = ctypes.CDLL(built_lib)
    missing = [n for n in declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_error_strings(built_lib):
    lib = ctypes.CDLL(built_lib)
    lib.ffv_error_string.restype = ctypes.c_char_p
    assert lib.ffv_error_string(0) == b"ok"
    assert b"balance" in lib.ffv_error_string(4)
