"""ctypes binding of the C ABI declared in include/ffv.h.

The shared library is built in-tree (forestfv_public_gb300/_lib/libffv.so, see build.py).
There is no fallback: if the library is missing or a CUDA device is unusable, loading or
context creation raises.
"""
from __future__ import annotations

import ctypes
import os

from .build import LIB

FFV_MAX_MATERIALS = 8
FFV_FP64 = 0
FFV_FP32_FLUX = 1
FFV_FLUX_REFERENCE = 0
FFV_FLUX_CONSISTENT = 1

ERRORS = {
    0: "ok", 1: "invalid argument", 2: "CUDA runtime error", 3: "mesh description rejected",
    4: "2:1 balance violated", 5: "non-finite residual or state on the device",
    6: "non-positive density on the device", 7: "bounded device wait ran out",
    8: "unsupported option", 9: "out of memory", 10: "call out of order",
}


class FFVError(RuntimeError):
    def __init__(self, code: int, what: str = ""):
        self.code = code
        super().__init__(f"{what}: {ERRORS.get(code, 'unknown error')} (code {code})")


class Params(ctypes.Structure):
    _fields_ = [("model", ctypes.c_int32), ("nmaterials", ctypes.c_int32),
                ("order", ctypes.c_int32), ("rk_steps", ctypes.c_int32),
                ("precision", ctypes.c_int32), ("prelax", ctypes.c_int32),
                ("gamma", ctypes.c_double * FFV_MAX_MATERIALS),
                ("pinf", ctypes.c_double * FFV_MAX_MATERIALS),
                ("mu", ctypes.c_double * FFV_MAX_MATERIALS),
                ("amin", ctypes.c_double), ("avf_lim", ctypes.c_double),
                ("zerou", ctypes.c_int32 * 3), ("flux_form", ctypes.c_int32),
                ("yield_", ctypes.c_double * FFV_MAX_MATERIALS)]


class ForestDesc(ctypes.Structure):
    _fields_ = [("ntrees", ctypes.c_int32 * 3), ("bc", ctypes.c_int32 * 6),
                ("tree_edge", ctypes.c_double)]


_lib = None

class TagParams(ctypes.Structure):
    """ffv_tag_params (include/ffv.h): the reference's refinement-criterion inputs."""
    _fields_ = [("uniform", ctypes.c_int32), ("lvl_uniform", ctypes.c_int32),
                ("grad_prs", ctypes.c_int32), ("lvl_prs", ctypes.c_int32),
                ("thr_prs", ctypes.c_double),
                ("grad_rho", ctypes.c_int32), ("lvl_rho", ctypes.c_int32),
                ("thr_rho", ctypes.c_double),
                ("grad_vel", ctypes.c_int32), ("lvl_vel", ctypes.c_int32),
                ("thr_vel", ctypes.c_double),
                ("inter0", ctypes.c_int32), ("lvl_inter0", ctypes.c_int32),
                ("lrs_inter0", ctypes.c_int32),
                ("inter1", ctypes.c_int32), ("lvl_inter1", ctypes.c_int32),
                ("lrs_inter1", ctypes.c_int32)]

    @classmethod
    def from_tuple(cls, t) -> "TagParams":
        """From (uniform, lvl, prs, lvl, thr, rho, lvl, thr, vel, lvl, thr, inter0, lvl,
        lrs, inter1, lvl, lrs), the order of the reference's input file lines."""
        names = [f[0] for f in cls._fields_]
        p = cls()
        for name, v in zip(names, t):
            setattr(p, name, float(v) if name.startswith("thr") else int(v))
        return p


EXPORTS = (
    "ffv_mesh_build", "ffv_mesh_build_part", "ffv_mesh_ncells", "ffv_mesh_free", "ffv_mesh_export", "ffv_create",
    "ffv_destroy", "ffv_set_mesh", "ffv_upload_state", "ffv_download_state", "ffv_stage",
    "ffv_step", "ffv_sync", "ffv_cfl_dt", "ffv_state_device_ptr", "ffv_launches_per_step",
    "ffv_error_string", "ffv_stream", "ffv_profile_stage", "ffv_stage_kernel_name", "ffv_step_async",
    "ffv_tags", "ffv_tags_raw", "ffv_tags_missed", "ffv_tags_smooth", "ffv_adapt", "ffv_adapt_map", "ffv_adapt_changes", "ffv_mesh_adapt", "ffv_mesh_leaves",
    "ffv_conservation_sums", "ffv_checkpoint_write", "ffv_checkpoint_info", "ffv_checkpoint_read", "ffv_restart_text_write",
    "ffv_restart_text_info", "ffv_restart_text_read", "ffv_tecplot_write", "ffv_export_fields",
    "ffv_mlp_create", "ffv_mlp_destroy", "ffv_mlp_get_params", "ffv_mlp_set_params",
    "ffv_mlp_set_norm", "ffv_mlp_fields", "ffv_mlp_features", "ffv_mlp_forward",
    "ffv_mlp_predict", "ffv_mlp_mark", "ffv_mlp_grad", "ffv_mlp_train",
)


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB):
        raise RuntimeError(f"{LIB} is not built; run forestfv_public_gb300.build.build() "
                           "(the CUDA library is required, there is no CPU path)")
    L = ctypes.CDLL(LIB)
    vp, i32, i64, dbl = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64, ctypes.c_double
    L.ffv_mesh_build.argtypes = [ctypes.POINTER(ForestDesc), i64, vp, vp, vp,
                                 ctypes.POINTER(vp), vp]
    L.ffv_mesh_build_part.argtypes = [ctypes.POINTER(ForestDesc), i64, vp, vp, vp,
                                      ctypes.POINTER(vp), vp]
    L.ffv_mesh_ncells.argtypes = [vp]
    L.ffv_mesh_ncells.restype = i64
    L.ffv_mesh_free.argtypes = [vp]
    L.ffv_mesh_free.restype = None
    L.ffv_mesh_export.argtypes = [vp] + [vp] * 10
    L.ffv_create.argtypes = [ctypes.POINTER(vp), ctypes.POINTER(Params), ctypes.c_int]
    L.ffv_destroy.argtypes = [vp]
    L.ffv_set_mesh.argtypes = [vp, vp]
    L.ffv_upload_state.argtypes = [vp, vp, i64, i32]
    L.ffv_download_state.argtypes = [vp, vp, i64, i32]
    L.ffv_stage.argtypes = [vp, i32, dbl]
    L.ffv_step.argtypes = [vp, dbl, i32]
    L.ffv_step_async.argtypes = [vp, dbl, i32]
    L.ffv_sync.argtypes = [vp]
    L.ffv_cfl_dt.argtypes = [vp, dbl, ctypes.POINTER(dbl)]
    L.ffv_state_device_ptr.argtypes = [vp, ctypes.POINTER(vp)]
    L.ffv_stream.argtypes = [vp, ctypes.POINTER(vp)]
    L.ffv_profile_stage.argtypes = [vp, i32, dbl, vp, i32, ctypes.POINTER(i32)]
    L.ffv_stage_kernel_name.argtypes = [vp, i32]
    L.ffv_stage_kernel_name.restype = ctypes.c_char_p
    L.ffv_launches_per_step.argtypes = [vp, ctypes.POINTER(i32)]
    L.ffv_tags.argtypes = [vp, vp, ctypes.POINTER(TagParams), vp, vp, vp]
    L.ffv_tags_raw.argtypes = [vp, vp, ctypes.POINTER(TagParams), vp, vp]
    L.ffv_tags_missed.argtypes = [vp, vp, ctypes.POINTER(TagParams), ctypes.POINTER(i64)]
    L.ffv_tags_smooth.argtypes = [vp, i32, vp]
    L.ffv_adapt.argtypes = [vp, vp, vp, ctypes.POINTER(vp)]
    L.ffv_mesh_leaves.argtypes = [vp, vp, vp, vp]
    L.ffv_adapt_map.argtypes = [vp, vp, vp, ctypes.POINTER(vp), vp]
    L.ffv_mesh_adapt.argtypes = [vp, vp, ctypes.POINTER(vp), vp]
    L.ffv_adapt_changes.argtypes = [vp, vp, ctypes.POINTER(i64), ctypes.POINTER(i64)]
    u64, f32 = ctypes.c_uint64, ctypes.c_float
    L.ffv_conservation_sums.argtypes = [vp, vp]
    cp = ctypes.c_char_p
    L.ffv_checkpoint_write.argtypes = [cp, vp, vp, i32, i64, dbl]
    L.ffv_checkpoint_info.argtypes = [cp, ctypes.POINTER(ForestDesc), ctypes.POINTER(i64),
                                      ctypes.POINTER(i32), ctypes.POINTER(i64), ctypes.POINTER(dbl)]
    L.ffv_checkpoint_read.argtypes = [cp, ctypes.POINTER(vp), vp]
    L.ffv_restart_text_write.argtypes = [cp, vp, vp, i32, i64, dbl]
    L.ffv_restart_text_info.argtypes = [cp, ctypes.POINTER(i64), ctypes.POINTER(i32),
                                        ctypes.POINTER(i64), ctypes.POINTER(dbl), ctypes.POINTER(i32)]
    L.ffv_restart_text_read.argtypes = [cp, ctypes.POINTER(ForestDesc), ctypes.POINTER(vp), vp]
    L.ffv_tecplot_write.argtypes = [cp, vp, i32, ctypes.POINTER(cp), vp, dbl]
    L.ffv_export_fields.argtypes = [vp, vp, ctypes.POINTER(i32)]
    L.ffv_mlp_create.argtypes = [ctypes.POINTER(vp), ctypes.c_int, u64]
    L.ffv_mlp_destroy.argtypes = [vp]
    L.ffv_mlp_get_params.argtypes = [vp, vp]
    L.ffv_mlp_set_params.argtypes = [vp, vp]
    L.ffv_mlp_set_norm.argtypes = [vp, vp, vp]
    L.ffv_mlp_fields.argtypes = [vp, vp]
    L.ffv_mlp_features.argtypes = [vp, vp, vp]
    L.ffv_mlp_forward.argtypes = [vp, vp, i64, vp]
    L.ffv_mlp_predict.argtypes = [vp, vp, vp]
    L.ffv_mlp_mark.argtypes = [vp, vp, f32, vp, i32]
    L.ffv_mlp_grad.argtypes = [vp, vp, vp, i64, vp, vp]
    L.ffv_mlp_train.argtypes = [vp, vp, vp, i64, i32, i32, f32, f32, u64, vp]
    L.ffv_error_string.argtypes = [ctypes.c_int]
    L.ffv_error_string.restype = ctypes.c_char_p
    _lib = L
    return L


def check(code: int, what: str) -> None:
    if code != 0:
        raise FFVError(code, what)
