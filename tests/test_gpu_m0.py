"""Model-0 CUDA path against the reference (golden fixtures) and the CPU restatement.

Tolerance: the plain FP64 form must match the reference's C code to 1e-12 relative L-inf
per conserved variable; the kernels round exactly as the reference does, so the tests
also require bit equality."""
import numpy as np
import pytest

from conftest import golden_names, load_golden
from helpers import mesh_from_golden, rel_linf

from forestfv_public_gb300 import FFVError, Mesh, Solver, leaves_from_paths
from forestfv_public_gb300.mesh import BC_REFLECTIVE, uniform_leaves
from oracle import pyoracle

pytestmark = pytest.mark.gpu
TOL = 1e-12


def run_gpu(mesh, S_aos, dt, steps, order=2, rk_steps=2, gamma=1.4, pinf=0.0):
    s = Solver(order=order, rk_steps=rk_steps, gamma=(gamma,), pinf=(pinf,))
    s.set_mesh(mesh)
    s.upload_state(np.ascontiguousarray(S_aos.T))
    s.step(dt, steps)
    out = s.download_state().T.copy()
    s.close()
    return out


@pytest.mark.parametrize("name", golden_names(model=0))
def test_gpu_matches_reference_fixture(name, built_lib):
    g = load_golden(name)
    m = mesh_from_golden(g)
    out = run_gpu(m, g["S_init"], float(g["dt"]), int(g["steps"]), int(g["order"]),
                  int(g["rk_steps"]), float(g["gamma"]), float(g["pinf"]))
    assert (rel_linf(out, g["S_final"]) <= TOL).all()
    assert np.array_equal(out, g["S_final"])


def test_stage_calls_equal_step(built_lib):
    g = load_golden("m0_sphere_amr")
    m = mesh_from_golden(g)
    dt = float(g["dt"])
    s = Solver()
    s.set_mesh(m)
    s.upload_state(g["S_init"].T.copy())
    for _ in range(int(g["steps"])):
        s.rk(0, dt)
        s.rk(1, dt)
        s.rk(2, dt)
    s.sync()
    out = s.download_state().T
    assert np.array_equal(out, g["S_final"])


def random_amr_leaves(rng, ntrees, base, top):
    """Refine around a random sphere, then split until 2:1 balanced (test helper)."""
    cells = {}
    lv = uniform_leaves(ntrees, base)
    for t, l, c in zip(lv.tree_ijk, lv.level, lv.cell_ijk):
        cells[(tuple(t), int(l), tuple(c))] = True
    ctr, rad = rng.uniform(0.3, 0.7, 3), rng.uniform(0.15, 0.3)
    edge = 1.0 / max(ntrees)

    def centre(t, l, c):
        h = edge / (1 << (l - 1))
        return np.array(t) * edge + (np.array(c) + 0.5) * h

    def split(key):
        t, l, c = key
        del cells[key]
        for k in range(8):
            off = ((k >> 1) & 1, k & 1, (k >> 2) & 1)
            cells[(t, l + 1, tuple(2 * np.array(c) + off))] = True

    for _ in range(top - base):
        for key in [k for k in cells if k[1] < top and np.linalg.norm(centre(*k) - ctr) < rad]:
            split(key)
    # 2:1 balance: split a leaf while a face neighbour's box holds a leaf two levels finer
    changed = True
    while changed:
        changed = False
        present = set()
        for (t, l, c) in cells:
            present.add((l, tuple(np.array(t) * (1 << (l - 1)) + np.array(c))))
        for key in list(cells):
            t, l, c = key
            g = np.array(t) * (1 << (l - 1)) + np.array(c)
            hit = False
            for ax in range(3):
                for d in (-1, 1):
                    q = g.copy()
                    q[ax] += d
                    for off in np.ndindex(4, 4, 4):
                        if (l + 2, tuple(q * 4 + np.array(off))) in present:
                            hit = True
                            break
                    if hit:
                        break
                if hit:
                    break
            if hit:
                split(key)
                changed = True
    keys = list(cells)
    tree = np.array([k[0] for k in keys], np.int32)
    lev = np.array([k[1] for k in keys], np.int32)
    cell = np.array([k[2] for k in keys], np.int32)
    from forestfv_public_gb300 import Leaves
    return Leaves(tree, lev, cell)


def smooth_state(cent, rng, gamma=1.4):
    k = rng.integers(1, 3, 3)
    ph = 2 * np.pi * (cent @ k)
    rho = 1.0 + 0.2 * np.sin(ph)
    u = 0.2 * np.cos(ph) + rng.uniform(-0.1, 0.1)
    v = 0.2 * np.sin(2 * ph + 0.3)
    w = -0.1 * np.sin(ph) * np.cos(ph)
    p = 1.0 + 0.3 * np.cos(ph)
    E = p / (gamma - 1.0) + 0.5 * rho * (u * u + v * v + w * w)
    return np.stack([rho, rho * u, rho * v, rho * w, E], axis=1)


@pytest.mark.parametrize("seed", [0, 1])
def test_gpu_matches_oracle_random_amr(seed, built_lib, oracle_lib):
    rng = np.random.default_rng(seed)
    lv = random_amr_leaves(rng, (2, 2, 2), 2, 4)
    bc = tuple(int(b) for b in rng.integers(1, 6, 6))
    m = Mesh((2, 2, 2), lv, bc=bc)
    S0 = smooth_state(m.centroids(), rng)
    rk = int(rng.integers(1, 5))
    ref = pyoracle.m0_advance(pyoracle.OracleMesh(m.export()), S0, 4e-4, 6, 2, rk)
    out = run_gpu(m, S0, 4e-4, 6, 2, rk)
    assert np.array_equal(out, ref)


def test_gpu_conservation_reflective_box(built_lib):
    """Size-independent property at 128^3: with reflective walls total mass and energy
    change only by rounding."""
    rng = np.random.default_rng(7)
    m = Mesh((4, 4, 4), uniform_leaves((4, 4, 4), 6), bc=(BC_REFLECTIVE,) * 6)
    S0 = smooth_state(m.centroids(), rng)
    out = run_gpu(m, S0, 1e-4, 10)
    for v in (0, 4):
        tot0, tot1 = S0[:, v].sum(), out[:, v].sum()
        assert abs(tot1 - tot0) <= 1e-12 * abs(tot0) * 10, (v, tot0, tot1)


def test_negative_density_is_reported(built_lib):
    """A negative density injected on the host into the uploaded state: the device status
    word reports FFV_ERR_NEG_DENSITY (the reference would run on into a NaN sound speed)."""
    g = load_golden("m0_sod_uniform")
    m = mesh_from_golden(g)
    S = g["S_init"].copy()
    S[17, 0] = -1.0
    s = Solver()
    s.set_mesh(m)
    s.upload_state(S.T.copy())
    with pytest.raises(FFVError) as e:
        s.step(1e-3, 1)
    assert e.value.code == 6
    s.close()


def test_nan_state_is_reported(built_lib):
    """A NaN injected on the host into the uploaded state: FFV_ERR_NAN from the status word
    (m0_residual.c:127-135 exits there)."""
    g = load_golden("m0_sod_uniform")
    m = mesh_from_golden(g)
    S = g["S_init"].copy()
    S[17, 4] = np.nan
    s = Solver()
    s.set_mesh(m)
    s.upload_state(S.T.copy())
    with pytest.raises(FFVError) as e:
        s.step(1e-3, 1)
    assert e.value.code == 5
    s.close()


def test_cfl_dt(built_lib):
    g = load_golden("m0_config1_sod32")
    m = mesh_from_golden(g)
    s = Solver()
    s.set_mesh(m)
    s.upload_state(g["S_init"].T.copy())
    dt = s.cfl_dt(0.4)
    assert abs(dt - float(g["dt"])) <= 1e-15 * dt
