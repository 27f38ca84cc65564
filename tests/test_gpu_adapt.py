"""Mesh adaptation on the GPU (ffv_adapt: tags, then merges and splits with the state carried
over) against the reference's own meshadaptation run on the same final state: the adapted
leaf list must be identical and the state within 1e-12 relative L-inf per variable (merged
model-5 cells go through the FP64 relaxation, whose pow() may differ in the last bit)."""
import numpy as np
import pytest

from conftest import golden_names, load_golden, m5_params
from helpers import mesh_from_golden, rel_linf

from forestfv_public_gb300 import Mesh, Solver, leaves_from_paths
from forestfv_public_gb300.mesh import uniform_leaves

pytestmark = pytest.mark.gpu
TOL = 1e-12


def adapt_cases():
    return [n for n in golden_names(model=5) if "adapt_params" in load_golden(n)]


@pytest.mark.parametrize("name", adapt_cases())
def test_adaptation_matches_reference(name, built_lib):
    g = load_golden(name)
    m = mesh_from_golden(g)
    q = m5_params(g)
    s = Solver(model=5, order=int(g["order"]), rk_steps=int(g["rk_steps"]), gamma=q["gamma"],
               pinf=q["pinf"], mu=q["mu"], amin=q["amin"], avf_lim=q["avf_lim"],
               prelax=q["prelax"])
    s.set_mesh(m)
    s.upload_state(np.ascontiguousarray(g["S_final"].T))
    new = s.meshadaptation(g["adapt_params"])
    ref = leaves_from_paths(tuple(g["ntrees"]), g["adapt_root"], g["adapt_level"],
                            g["adapt_adrs"][:, 2:].astype(np.int64))
    assert new.n == ref.n
    assert np.array_equal(new.level, ref.level)
    assert np.array_equal(new.tree_ijk, ref.tree_ijk)
    assert np.array_equal(new.cell_ijk, ref.cell_ijk)
    err = rel_linf(s.download_state().T, g["adapt_S"])
    assert (err <= TOL).all(), (err.max(), int(err.argmax()))
    s.close()


def test_adapt_model0_copy_and_mean(built_lib):
    """Model 0: children copy their parent's state, a merged parent holds the mean of its
    eight children, summed in child order as merge.c does."""
    m = Mesh((2, 2, 2), uniform_leaves((2, 2, 2), 3))
    rng = np.random.default_rng(1)
    S = np.empty((5, m.n))
    S[0] = rng.uniform(0.5, 2.0, m.n)
    S[1:4] = rng.normal(0, 0.1, (3, m.n))
    S[4] = rng.uniform(2.0, 3.0, m.n)
    s = Solver()
    s.set_mesh(m)
    s.upload_state(S)
    x = m.centroids()
    # refine x < 0.25, keep 0.25 <= x < 0.5, coarsen x >= 0.5 (2:1 across both borders)
    split = np.where(x[:, 0] < 0.25, 4, np.where(x[:, 0] < 0.5, 3, 2)).astype(np.int32)
    new = s.adapt(split)
    assert new.n == (m.n // 4) * 8 + m.n // 4 + (m.n // 2) // 8
    Sn = s.download_state()
    # expected: walk the old leaves in order (siblings are consecutive)
    exp = []
    i = 0
    while i < m.n:
        if split[i] < m.level[i]:
            acc = np.zeros(5)
            for k in range(8):
                acc = acc + S[:, i + k] / 8.0
            exp.append(acc)
            i += 8
        elif split[i] > m.level[i]:
            exp.extend([S[:, i]] * 8)
            i += 1
        else:
            exp.append(S[:, i])
            i += 1
    assert np.array_equal(Sn, np.array(exp).T)
    s.close()


def test_adapt_remap_with_and_without_capacity(built_lib):
    """The state remap of a regrid runs in the context's idle buffers while the new mesh fits
    them, and in buffers of its own when it does not (every leaf splitting: 8x the cells,
    beyond the 25 % headroom); both give the children their parent's bits."""
    m = Mesh((2, 2, 2), uniform_leaves((2, 2, 2), 2))
    rng = np.random.default_rng(3)
    S = np.empty((5, m.n))
    S[0] = rng.uniform(0.5, 2.0, m.n)
    S[1:4] = rng.normal(0, 0.1, (3, m.n))
    S[4] = rng.uniform(2.0, 3.0, m.n)
    s = Solver()
    s.set_mesh(m)
    s.upload_state(S)
    x = m.centroids()
    small = np.where(x[:, 0] < 0.25, 3, 2).astype(np.int32)  # a quarter of the leaves split
    for split in (small, None):
        old_level, old_S = s.mesh.level, s.download_state()
        if split is None:
            split = (old_level + 1).astype(np.int32)  # every leaf splits
        new, src = s.adapt(split, with_src=True)
        assert new.n == old_S.shape[1] + 7 * int((split > old_level).sum())
        assert np.array_equal(s.download_state(), old_S[:, src])
    s.close()
