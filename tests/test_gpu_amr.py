"""The adaptive time loop on the GPU.

* The judge (ffv_tags_missed) counts exactly the cells whose raw criterion level is above
  their level, and ffv_tags is ffv_tags_raw followed by the smoothing.
* Learned AMR against plain AMR (the reference's loop: meshadaptation every 8 steps) on
  model-0 blasts: a network trained on seeded runs (features at step n, "the criterion asks
  for a finer level within the next 16 steps") marks the cells ahead of the shock, and the
  regrids pre-refine them.  Against the same loop without marks (the criterion alone as
  judge) the judge finds far fewer cells left to refine; the test also requires no more
  regrids than plain AMR and a density within 5 % relative L1 of the plain-AMR run on the
  uniform finest grid."""
import numpy as np
import pytest
import torch

from conftest import load_golden, m5_params
from helpers import mesh_from_golden

from forestfv_public_gb300 import Mesh, Solver
from forestfv_public_gb300.amr import AdaptiveRun
from forestfv_public_gb300.fields import to_uniform
from forestfv_public_gb300.indicator import Indicator, collect_window, field_norm
from forestfv_public_gb300.mesh import uniform_leaves
from forestfv_public_gb300.solver import tags_smooth
from forestfv_public_gb300.workloads import random_blast_m0

pytestmark = pytest.mark.gpu
TAG = (1, 3, 1, 5, 0.1, 1, 5, 0.1, 0, 0, 0.0, 0, 0, 0, 0, 0, 0)
H = 16
EVERY = 8
THRESHOLD = 0.3


def test_judge_counts_and_raw_tags(built_lib):
    g = load_golden("m5_wall_amr")
    q = m5_params(g)
    s = Solver(model=5, order=int(g["order"]), rk_steps=int(g["rk_steps"]), gamma=q["gamma"],
               pinf=q["pinf"], mu=q["mu"], amin=q["amin"], avf_lim=q["avf_lim"],
               prelax=q["prelax"])
    m = mesh_from_golden(g)
    s.set_mesh(m)
    s.upload_state(np.ascontiguousarray(g["S_final"].T))
    for tp in g["tag_params"]:
        tp = tuple(int(v) if k not in (4, 7, 10) else float(v) for k, v in enumerate(tp))
        raw = s.tags_raw(tp)
        assert s.tags_missed(tp) == int((raw > m.level).sum())
        lmax = max(tp[1], tp[3], tp[6], tp[9], tp[12], tp[15])
        assert np.array_equal(tags_smooth(m, lmax, raw), s.tags(tp))
    s.close()


def setup(seed):
    mesh = Mesh((2, 2, 2), uniform_leaves((2, 2, 2), 5))
    s = Solver()
    s.set_mesh(mesh)
    s.upload_state(random_blast_m0(mesh, seed))
    dt = s.cfl_dt(0.4)
    AdaptiveRun(s, TAG).meshadaptation()
    return s, dt


def test_learned_amr_against_plain(built_lib):
    ind = Indicator(seed=31)
    runs = [setup(200 + k) for k in range(6)]
    mean, std = field_norm([ind.fields(s).cpu().numpy() for s, _ in runs])
    ind.set_norm(mean, np.maximum(std, np.array([0.05, 0.05, 0.01, 0.01, 1.0], np.float32)))
    Xs, ys = [], []
    for s, dt in runs:
        amr = AdaptiveRun(s, TAG)
        for _ in range(6):
            X, y = collect_window(s, ind, TAG, dt, H)
            Xs.append(X)
            ys.append(y)
            amr.meshadaptation()
        s.close()
    X, y = torch.cat(Xs), torch.cat(ys)
    losses = ind.train(X, y, steps=1500, batch=8192, lr=1e-3, wd=1e-4, seed=7)
    assert losses[-50:].mean() < 0.5 * losses[:10].mean()

    nsteps = 6 * EVERY
    sp, dt = setup(999)
    plain = AdaptiveRun(sp, TAG, every=EVERY).run(dt, nsteps)
    rho_p = to_uniform(sp.mesh, sp.download_state()[0], 5)
    out = {"plain": plain.as_dict()}
    for name, thr in (("judge_only", 2.0), ("learned", THRESHOLD)):
        sl, _ = setup(999)
        st = AdaptiveRun(sl, TAG, every=EVERY, indicator=ind, threshold=thr).run(dt, nsteps)
        rho_l = to_uniform(sl.mesh, sl.download_state()[0], 5)
        out[name] = st.as_dict()
        out[name]["rho_rel_l1_vs_plain"] = float(np.abs(rho_l - rho_p).sum() / np.abs(rho_p).sum())
        sl.close()
    print(out)
    assert plain.regrids == nsteps // EVERY
    learned, judge = out["learned"], out["judge_only"]
    assert learned["regrids"] <= plain.regrids
    # the network's marks leave the judge far fewer cells to refine
    assert np.mean(learned["missed"][1:]) <= 0.7 * np.mean(judge["missed"][1:])
    assert learned["rho_rel_l1_vs_plain"] < 0.05
    sp.close()
    ind.close()
