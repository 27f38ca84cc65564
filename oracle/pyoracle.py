"""ctypes binding of the CPU restatement (oracle/_build/libffv_oracle.so).

TEST INFRASTRUCTURE: the oracle for the CUDA path, used only by tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libffv_oracle.so")

_lib = None


class _Mesh(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int64)] + [(k, ctypes.c_void_p) for k in (
        "bc", "nn", "neigfc", "nb", "area", "nrm", "dist_cf", "dist_cc", "vol", "si")]


class _Params(ctypes.Structure):
    _fields_ = [("order", ctypes.c_int32), ("rk_steps", ctypes.c_int32),
                ("gamma", ctypes.c_double), ("pinf", ctypes.c_double)]


class _M5Params(ctypes.Structure):
    _fields_ = [("nmat", ctypes.c_int32), ("order", ctypes.c_int32), ("rk_steps", ctypes.c_int32),
                ("prelax", ctypes.c_int32), ("zerou", ctypes.c_int32 * 3),
                ("flux_form", ctypes.c_int32), ("gamma", ctypes.c_double * 4),
                ("pinf", ctypes.c_double * 4), ("mu", ctypes.c_double * 4),
                ("amin", ctypes.c_double), ("avf_lim", ctypes.c_double),
                ("yield_", ctypes.c_double * 4)]


def build() -> str:
    srcs = sorted(os.path.join(HERE, f) for f in os.listdir(HERE) if f.endswith(".c"))
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    cmd = ["gcc", "-std=c99", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
           "-o", LIB, *srcs, "-lm"]
    subprocess.run(cmd, check=True, capture_output=True)
    return LIB


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = ctypes.CDLL(LIB)
        L.ffvo_m0_advance.argtypes = [ctypes.POINTER(_Mesh), ctypes.POINTER(_Params),
                                      ctypes.c_void_p, ctypes.c_double, ctypes.c_int]
        L.ffvo_m5_advance.argtypes = [ctypes.POINTER(_Mesh), ctypes.POINTER(_M5Params),
                                      ctypes.c_void_p, ctypes.c_double, ctypes.c_int]
        L.ffvo_m5_gfm_calls.restype = ctypes.c_long
        L.ffvo_m5_gfm_calls.argtypes = [ctypes.c_int]
        _lib = L
    return _lib


def m5_gfm_calls() -> tuple[int, int]:
    """(m5_gfm, m5_gfm_rel) invocations of the model-5 restatement in this process."""
    return int(lib().ffvo_m5_gfm_calls(0)), int(lib().ffvo_m5_gfm_calls(1))


class OracleMesh:
    """Reference-form geometry (keys as Mesh.export() / the reference dump)."""

    def __init__(self, g: dict, si=None):
        self._keep = {}

        def P(name, a, dt):
            a = np.ascontiguousarray(a, dtype=dt)
            self._keep[name] = a
            return a.ctypes.data

        n = int(np.asarray(g["vol"]).shape[0])
        self.n = n
        self.c = _Mesh(n=n, bc=P("bc", g["bc"], np.int32), nn=P("nn", g["nn"], np.int32),
                       neigfc=P("neigfc", g["neigfc"], np.int32), nb=P("nb", g["nb"], np.int32),
                       area=P("area", g["area"], np.float64), nrm=P("nrm", g["nrm"], np.float64),
                       dist_cf=P("dist_cf", g["dist_cf"], np.float64),
                       dist_cc=P("dist_cc", g["dist_cc"], np.float64),
                       vol=P("vol", g["vol"], np.float64),
                       si=P("si", np.zeros(n) if si is None else si, np.int32))


def m0_advance(mesh: OracleMesh, S_aos: np.ndarray, dt: float, nsteps: int, order: int = 2,
               rk_steps: int = 2, gamma: float = 1.4, pinf: float = 0.0) -> np.ndarray:
    """Advance an AoS [n,5] state; returns the new state (input untouched)."""
    S = np.ascontiguousarray(S_aos, dtype=np.float64).copy()
    p = _Params(order=order, rk_steps=rk_steps, gamma=gamma, pinf=pinf)
    err = lib().ffvo_m0_advance(ctypes.byref(mesh.c), ctypes.byref(p), S.ctypes.data, dt, nsteps)
    if err:
        raise RuntimeError(f"oracle stopped with code {err} (the reference would exit here)")
    return S


def m5_advance(mesh: OracleMesh, S_aos: np.ndarray, dt: float, nsteps: int, m5: dict,
               order: int = 2, rk_steps: int = 2, zerou=(0, 0, 0)) -> np.ndarray:
    """Model 5: advance an AoS [n, 3N+12] state; returns the new state."""
    S = np.ascontiguousarray(S_aos, dtype=np.float64).copy()
    p = _M5Params(nmat=len(m5["gamma"]), order=order, rk_steps=rk_steps, prelax=m5["prelax"],
                  amin=m5["amin"], avf_lim=m5["avf_lim"], flux_form=m5.get("flux_form", 0))
    p.zerou[:] = zerou
    for i, (g, q, mu) in enumerate(zip(m5["gamma"], m5["pinf"], m5["mu"])):
        p.gamma[i], p.pinf[i], p.mu[i] = g, q, mu
    for i, y in enumerate(m5.get("yield", ())):
        p.yield_[i] = y
    err = lib().ffvo_m5_advance(ctypes.byref(mesh.c), ctypes.byref(p), S.ctypes.data, dt, nsteps)
    if err:
        raise RuntimeError(f"oracle stopped with code {err} (the reference would exit here)")
    return S
