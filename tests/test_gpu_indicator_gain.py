"""What the trained indicator gains over the plain criterion alone.

Setting: model-0 spherical blasts on the 32^3 forest (CFL 0.4), the relative-jump
criterion (pressure and density, threshold 0.1, one level above the mesh), horizon 8
steps.  The network is trained on seeded runs (pairs of features at step n and the
criterion's verdict at step n + 8) and evaluated on a run it has not seen: of the cells the
criterion will flag 8 steps later, the criterion flags at step n only those the shock has
already reached; the network, evaluated at step n, marks the cells ahead of it.  The test
requires the combination to cover clearly more of the future flags than the criterion
alone, with a bounded number of extra cells."""
import numpy as np
import pytest
import torch

from forestfv_public_gb300 import Mesh, Solver
from forestfv_public_gb300.indicator import Indicator, collect, field_norm, gain_report
from forestfv_public_gb300.mesh import uniform_leaves
from forestfv_public_gb300.workloads import random_blast_m0

pytestmark = pytest.mark.gpu
TAG = (1, 4, 1, 5, 0.1, 1, 5, 0.1, 0, 0, 0.0, 0, 0, 0, 0, 0, 0)
H = 8


def run(mesh, seed):
    s = Solver()
    s.set_mesh(mesh)
    s.upload_state(random_blast_m0(mesh, seed))
    return s, s.cfl_dt(0.4)


def test_indicator_gain_over_criterion(built_lib):
    mesh = Mesh((4, 4, 4), uniform_leaves((4, 4, 4), 4))
    ind = Indicator(seed=21)
    runs = [run(mesh, 100 + k) for k in range(6)]
    F = [ind.fields(s).cpu().numpy() for s, _ in runs]
    mean, std = field_norm(F)
    ind.set_norm(mean, np.maximum(std, np.array([0.05, 0.05, 0.01, 0.01, 1.0], np.float32)))
    Xs, ys = [], []
    for s, dt in runs:
        X, y, _, _ = collect(s, ind, TAG, dt, snapshots=6, every=H, horizon=H)
        Xs.append(X)
        ys.append(y)
        s.close()
    X, y = torch.cat(Xs), torch.cat(ys)
    losses = ind.train(X, y, steps=1500, batch=8192, lr=1e-3, wd=1e-4, seed=5)
    assert losses[-50:].mean() < 0.5 * losses[:10].mean()
    s, dt = run(mesh, 999)
    rep = gain_report(ind, s, TAG, dt, snapshots=5, every=H, horizon=H)
    s.close()
    ind.close()
    print(rep)
    assert rep["coverage_criterion"] < 0.9
    assert rep["coverage_criterion_and_network"] >= rep["coverage_criterion"] + 0.1
    assert rep["cells_marked_criterion_and_network"] <= 3 * rep["cells_marked_criterion"]
