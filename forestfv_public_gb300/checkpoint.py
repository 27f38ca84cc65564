"""Checkpoint/restart and field export (host side), over csrc/ffv_io.cpp.

  save_checkpoint / load_checkpoint   binary, Morton-keyed leaves + FP64 state, bit-exact
  write_restart_text / read_restart_text
                                      the reference's text restart (restart_save.c:13-50,
                                      restart_load.c:13-45), byte-identical on write
  write_tecplot                       Tecplot ASCII of per-leaf fields (the kind of file
                                      m5_exportfield_linked.c writes), headless
  export_fields                       the derived per-leaf fields of a solver's state,
                                      computed on the device (ffv_export_fields)
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .mesh import Mesh


def _desc_tuple(d) -> tuple:
    return tuple(d.ntrees), tuple(d.bc), float(d.tree_edge)


def save_checkpoint(path: str, mesh: Mesh, S: np.ndarray, istep: int = 0, time: float = 0.0) -> None:
    S = np.ascontiguousarray(S, dtype=np.float64)
    assert S.ndim == 2 and S.shape[1] == mesh.n
    _lib.check(_lib.lib().ffv_checkpoint_write(str(path).encode(), mesh.handle, S.ctypes.data,
                                               S.shape[0], int(istep), float(time)),
               "ffv_checkpoint_write")


def checkpoint_info(path: str) -> dict:
    d = _lib.ForestDesc()
    n, neq, istep, t = ctypes.c_int64(), ctypes.c_int32(), ctypes.c_int64(), ctypes.c_double()
    _lib.check(_lib.lib().ffv_checkpoint_info(str(path).encode(), ctypes.byref(d), ctypes.byref(n),
                                              ctypes.byref(neq), ctypes.byref(istep),
                                              ctypes.byref(t)), "ffv_checkpoint_info")
    ntrees, bc, edge = _desc_tuple(d)
    return {"n": n.value, "neq": neq.value, "istep": istep.value, "time": t.value,
            "ntrees": ntrees, "bc": bc, "tree_edge": edge}


def load_checkpoint(path: str):
    """Returns (Mesh, S [neq, n] in the mesh's cell order, istep, time)."""
    info = checkpoint_info(path)
    S = np.empty((info["neq"], info["n"]))
    h = ctypes.c_void_p()
    _lib.check(_lib.lib().ffv_checkpoint_read(str(path).encode(), ctypes.byref(h), S.ctypes.data),
               "ffv_checkpoint_read")
    mesh = Mesh.from_handle(h, info["ntrees"], info["bc"], info["tree_edge"])
    return mesh, S, info["istep"], info["time"]


def write_restart_text(path: str, mesh: Mesh, S: np.ndarray, istep: int = 0,
                       time: float = 0.0) -> None:
    S = np.ascontiguousarray(S, dtype=np.float64)
    assert S.ndim == 2 and S.shape[1] == mesh.n
    _lib.check(_lib.lib().ffv_restart_text_write(str(path).encode(), mesh.handle, S.ctypes.data,
                                                 S.shape[0], int(istep), float(time)),
               "ffv_restart_text_write")


def read_restart_text(path: str, ntrees, bc=(2,) * 6, tree_edge: float | None = None):
    """The reference's restart file on the forest of ntrees[0] x ntrees[1] x ntrees[2] trees:
    returns (Mesh, S [neq, n] in the mesh's cell order, istep, time)."""
    n, neq, istep = ctypes.c_int64(), ctypes.c_int32(), ctypes.c_int64()
    t, nt = ctypes.c_double(), ctypes.c_int32()
    L = _lib.lib()
    _lib.check(L.ffv_restart_text_info(str(path).encode(), ctypes.byref(n), ctypes.byref(neq),
                                       ctypes.byref(istep), ctypes.byref(t), ctypes.byref(nt)),
               "ffv_restart_text_info")
    d = _lib.ForestDesc()
    d.ntrees[:] = tuple(int(x) for x in ntrees)
    d.bc[:] = tuple(int(b) for b in bc)
    d.tree_edge = float(tree_edge if tree_edge is not None else 1.0 / max(ntrees))
    S = np.empty((neq.value, n.value))
    h = ctypes.c_void_p()
    _lib.check(L.ffv_restart_text_read(str(path).encode(), ctypes.byref(d), ctypes.byref(h),
                                       S.ctypes.data), "ffv_restart_text_read")
    mesh = Mesh.from_handle(h, tuple(d.ntrees), tuple(d.bc), d.tree_edge)
    return mesh, S, istep.value, t.value


def write_tecplot(path: str, mesh: Mesh, fields: dict, time: float = 0.0) -> None:
    names = list(fields)
    F = np.ascontiguousarray(np.stack([np.asarray(fields[k], np.float64) for k in names])
                             if names else np.zeros((0, mesh.n)))
    arr = (ctypes.c_char_p * max(1, len(names)))(*[k.encode() for k in names])
    _lib.check(_lib.lib().ffv_tecplot_write(str(path).encode(), mesh.handle, len(names), arr,
                                            F.ctypes.data, float(time)), "ffv_tecplot_write")


def field_names(model: int, nmat: int = 1) -> list[str]:
    if model == 5:
        return (["rho", "u", "v", "w", "p"] + [f"alpha{k}" for k in range(nmat)]
                + [f"p{k}" for k in range(nmat)] + ["von_mises"])
    return ["rho", "u", "v", "w", "p"]


def export_fields(solver) -> dict:
    """The solver's per-leaf fields (ffv_export_fields, on the device), as host arrays."""
    import torch
    nf = ctypes.c_int32()
    L = _lib.lib()
    _lib.check(L.ffv_export_fields(solver._h, None, ctypes.byref(nf)), "ffv_export_fields")
    F = torch.empty((nf.value, solver.mesh.n), dtype=torch.float64,
                    device=f"cuda:{solver.device}")
    _lib.check(L.ffv_export_fields(solver._h, ctypes.c_void_p(F.data_ptr()), ctypes.byref(nf)),
               "ffv_export_fields")
    Fh = F.cpu().numpy()
    names = field_names(solver.params.model, solver.params.nmaterials)
    return {k: Fh[i] for i, k in enumerate(names)}
