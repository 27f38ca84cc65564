"""The split step's data path on the GPU: two ranks emulated in one process on one GPU, each
a Solver on its part of the forest (ffv_mesh_build_part: own cells and a halo of
3 x rk_steps face hops), the halo exchange after every step done by device copies along the
same plan the NCCL exchange follows (forestfv_public_gb300/partition.py).  The ranks' own cells
must equal the single-GPU step bit for bit."""
import numpy as np
import pytest
import torch

import bench
from forestfv_public_gb300 import Solver
from forestfv_public_gb300 import partition as P
from forestfv_public_gb300.mesh import Leaves

pytestmark = pytest.mark.gpu
STEPS = 3


@pytest.mark.parametrize("workload,precision", [("config3", 0), ("config3", 1), ("config2", 0),
                                                ("config1", 0)])
def test_split_step_equals_single_gpu(workload, precision, built_lib):
    mesh, S0, dt, _, kw, _, _ = bench.WORKLOADS[workload](small=True)
    kw = dict(kw, precision=precision)
    if kw.get("model", 0) == 5:
        kw["flux_form"] = 1
    ref = Solver(**kw)
    ref.set_mesh(mesh)
    ref.upload_state(S0)
    ref.step(dt, STEPS)
    want = ref.download_state()
    ref.close()
    plans = P.plan(mesh.export(), 2, P.HALO_HOPS_PER_STAGE * kw.get("rk_steps", 2))
    leaves = Leaves(mesh.tree_ijk, mesh.level, mesh.cell_ijk)
    ranks = [P.RankStep(mesh.ntrees, leaves, mesh.bc, p, kw) for p in plans]
    for r in ranks:
        r.upload(S0)
    for _ in range(STEPS):
        for r in ranks:
            r.solver.step(dt, 1)
        states = [r.state() for r in ranks]
        for p, S in zip(plans, states):
            for q, pos in p.recv.items():
                src = torch.as_tensor(plans[q].send[p.rank], device=S.device)
                S[:, torch.as_tensor(pos, device=S.device)] = states[q][:, src]
        torch.cuda.synchronize()
    got = np.empty_like(want)
    for r in ranks:
        a, b = r.plan.own
        got[:, a:b] = r.own_state()
        r.close()
    assert np.array_equal(got, want)
