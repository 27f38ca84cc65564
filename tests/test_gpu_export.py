"""Field export and restart on the GPU.

* ffv_export_fields against the host restatement of the reference's equation of state
  (fields.primitives, float64 numpy) on fixture states of both models.
* A run stopped, written to a binary checkpoint, read back and continued gives the same
  bits as the uninterrupted run."""
import numpy as np
import pytest

from conftest import load_golden, m5_params
from helpers import mesh_from_golden

from forestfv_public_gb300 import Solver
from forestfv_public_gb300.checkpoint import export_fields, load_checkpoint, save_checkpoint
from forestfv_public_gb300.fields import primitives

pytestmark = pytest.mark.gpu


def m5_solver(g):
    q = m5_params(g)
    return Solver(model=5, order=int(g["order"]), rk_steps=int(g["rk_steps"]), gamma=q["gamma"],
                  pinf=q["pinf"], mu=q["mu"], amin=q["amin"], avf_lim=q["avf_lim"],
                  prelax=q["prelax"]), q


def close(a, b, tol):
    return np.abs(a - b).max() <= tol * max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("name", ["m5_wall_amr", "m5_bubble_prelax3"])
def test_export_fields_model5(name, built_lib):
    g = load_golden(name)
    s, q = m5_solver(g)
    m = mesh_from_golden(g)
    s.set_mesh(m)
    S = np.ascontiguousarray(g["S_final"].T)
    s.upload_state(S)
    F = export_fields(s)
    ref = primitives(S, q["gamma"], q["pinf"], q["mu"], q["amin"])
    N = len(q["gamma"])
    assert close(F["rho"], ref["rho"], 1e-13)
    assert close(F["p"], ref["p"], 1e-9)
    for k in range(N):
        assert close(F[f"alpha{k}"], ref["alpha"][k], 1e-13)
    assert close(F["von_mises"], ref["vm"], 1e-7)
    u = -S[N:N + 3] / ref["rho"]
    assert close(np.stack([F["u"], F["v"], F["w"]]), u, 1e-13)
    s.close()


def test_export_fields_model0(built_lib):
    g = load_golden("m0_sphere_amr")
    s = Solver(gamma=(float(g["gamma"]),), pinf=(float(g["pinf"]),))
    m = mesh_from_golden(g)
    s.set_mesh(m)
    S = np.ascontiguousarray(g["S_final"].T)
    s.upload_state(S)
    F = export_fields(s)
    rho = S[0]
    u = -S[1:4] / rho
    e = S[4] / rho - 0.5 * (u * u).sum(axis=0)
    p = rho * (float(g["gamma"]) - 1.0) * e - float(g["gamma"]) * float(g["pinf"])
    assert close(F["rho"], rho, 0) and close(np.stack([F["u"], F["v"], F["w"]]), u, 1e-14)
    assert close(F["p"], p, 1e-12)
    s.close()


def test_checkpoint_continue_bit_exact(tmp_path, built_lib):
    g = load_golden("m5_wall_gfm")
    s, _ = m5_solver(g)
    m = mesh_from_golden(g)
    s.set_mesh(m)
    s.upload_state(np.ascontiguousarray(g["S_init"].T))
    dt = float(g["dt"])
    s.step(dt, 2)
    p = str(tmp_path / "c.ffvc")
    save_checkpoint(p, s.mesh, s.download_state(), istep=2, time=2 * dt)
    s.step(dt, 2)
    straight = s.download_state()
    m2, S2, istep, t = load_checkpoint(p)
    r, _ = m5_solver(g)
    r.set_mesh(m2)
    r.upload_state(S2)
    r.step(dt, 2)
    assert istep == 2
    assert np.array_equal(r.download_state().view(np.uint64), straight.view(np.uint64))
    s.close()
    r.close()
