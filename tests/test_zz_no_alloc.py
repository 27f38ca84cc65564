"""ffv_step_noalloc (the model-0 step that allocates nothing) against ffv_step.

The entry point is called through the C ABI with the state in device memory that the test
owns; its results must equal ffv_step's on the same inputs within the tolerance of the
model-0 tests (1e-12 relative L-inf per conserved variable; both run the same kernels, so
the test also requires bit equality), over two calls in a row.  Named to be collected last,
so that it runs both alone and after every other test in one process."""
import ctypes

import numpy as np
import pytest

from conftest import load_golden
from helpers import mesh_from_golden, rel_linf

from forestfv_public_gb300 import Mesh, Solver, _lib
from forestfv_public_gb300.mesh import uniform_leaves

TOL = 1e-12
FFV_ERR_UNSUPPORTED = 8
FFV_ERR_TOO_LARGE = 11


def noalloc_fn(built_lib):
    L = ctypes.CDLL(built_lib)
    f = L.ffv_step_noalloc
    f.argtypes = [ctypes.c_void_p, ctypes.POINTER(_lib.Params), ctypes.c_void_p,
                  ctypes.c_double, ctypes.c_int32, ctypes.c_void_p]
    f.restype = ctypes.c_int
    return f


def params(order=2, rk_steps=2, gamma=1.4, pinf=0.0, model=0):
    p = _lib.Params()
    p.model, p.nmaterials, p.order, p.rk_steps, p.precision = model, 1, order, rk_steps, 0
    p.gamma[0], p.pinf[0] = gamma, pinf
    return p


def case(name):
    g = load_golden(name)
    return (mesh_from_golden(g), g["S_init"], float(g["dt"]),
            params(int(g["order"]), int(g["rk_steps"]), float(g["gamma"]), float(g["pinf"])))


class Pair:
    """The same problem advanced by ffv_step (a context) and by ffv_step_noalloc (a torch
    device tensor owned by the test)."""

    def __init__(self, f, mesh, S_aos, p):
        import torch
        self.torch, self.f, self.mesh, self.p = torch, f, mesh, p
        self.ref = Solver(order=p.order, rk_steps=p.rk_steps, gamma=(p.gamma[0],),
                          pinf=(p.pinf[0],))
        self.ref.set_mesh(mesh)
        self.ref.upload_state(np.ascontiguousarray(S_aos.T))
        self.d_S = torch.from_numpy(np.ascontiguousarray(S_aos.T)).to("cuda:0")

    def advance(self, dt, nsteps):
        self.ref.step(dt, nsteps)
        stream = self.torch.cuda.current_stream(0).cuda_stream
        rc = self.f(self.mesh.handle, ctypes.byref(self.p), self.d_S.data_ptr(), dt, nsteps,
                    stream)
        assert rc == 0, _lib.lib().ffv_error_string(rc)
        got = self.d_S.cpu().numpy().T
        want = self.ref.download_state().T
        assert (rel_linf(got, want) <= TOL).all()
        assert np.array_equal(got, want)

    def close(self):
        self.ref.close()


@pytest.mark.gpu
def test_noalloc_two_calls_match_step(built_lib):
    """AMR mesh with coarse/fine faces: two calls in a row, each against ffv_step."""
    f = noalloc_fn(built_lib)
    mesh, S0, dt, p = case("m0_sphere_amr")
    pr = Pair(f, mesh, S0, p)
    pr.advance(dt, 4)
    pr.advance(dt, 3)
    pr.close()


@pytest.mark.gpu
def test_noalloc_consecutive_meshes_and_schemes(built_lib):
    """Consecutive calls on different meshes, orders and RK schemes: nothing of the
    previous call's scratch contents leaks into the next."""
    f = noalloc_fn(built_lib)
    cases = [case(nm) for nm in
             ("m0_blast_amr_deep", "m0_wave_order1_rk3_reflective", "m0_stiff_rk4_allbc")]
    pairs = [Pair(f, mesh, S0, p) for mesh, S0, _, p in cases]
    for rep in range(2):
        for pr, (_, _, dt, _) in zip(pairs, cases):
            pr.advance(dt, 2 + rep)
    for pr in pairs:
        pr.close()


def test_noalloc_rejects_oversized_and_unsupported(built_lib):
    """Size and option checks come before any device work (no GPU needed)."""
    f = noalloc_fn(built_lib)
    big = Mesh((4, 4, 4), uniform_leaves((4, 4, 4), 5))  # 64^3 = 262144 cells > 65536
    assert big.n > 65536
    dummy = ctypes.c_void_p(16)  # never dereferenced: the checks return first
    assert f(big.handle, ctypes.byref(params()), dummy, 1e-3, 1, None) == FFV_ERR_TOO_LARGE
    small = Mesh((2, 2, 2), uniform_leaves((2, 2, 2), 2))
    assert f(small.handle, ctypes.byref(params(model=5)), dummy, 1e-3, 1, None) == \
        FFV_ERR_UNSUPPORTED
    p32 = params()
    p32.precision = 1
    assert f(small.handle, ctypes.byref(p32), dummy, 1e-3, 1, None) == FFV_ERR_UNSUPPORTED
