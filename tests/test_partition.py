"""The split step on CPU ranks (gloo, world sizes 2 and 3): contiguous Morton ranges, halos of
3 x rk_steps face hops, one halo exchange per time step (forestfv_public_gb300/partition.py).
Each rank advances its part -- its own cells and the halo, as a mesh of its own -- with the CPU
restatement standing in for the GPU step; after the steps the ranks' own cells, gathered,
must equal the single-rank run bit for bit."""
import os
import socket
import sys

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
STEPS = 3


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _case(workload):
    sys.path.insert(0, ROOT)
    import bench
    from oracle.forest import Forest
    F, state, dt, kw, _ = bench.cpu_case(workload)
    S0 = state(F.centroids())
    return F, S0, dt, kw


def _advance(geo, S, dt, kw, steps, flux_form=1):
    sys.path.insert(0, ROOT)
    import bench
    from oracle import pyoracle
    om = pyoracle.OracleMesh(geo)
    return bench._cpu_advance(om, np.ascontiguousarray(S.T), dt, steps, kw, flux_form).T


def _rank(rank, world, port, workload, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    from forestfv_public_gb300 import partition as P
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        F, S0, dt, kw = _case(workload)
        plans = P.plan(F.geometry(), world, P.HALO_HOPS_PER_STAGE * kw.get("rk_steps", 2))
        p = plans[rank]
        geo = F.geometry(p.cells)
        S = torch.from_numpy(np.ascontiguousarray(S0[:, p.cells]))
        for _ in range(STEPS):
            S = torch.from_numpy(np.ascontiguousarray(_advance(geo, S.numpy(), dt, kw, 1)))
            P.exchange(S, p)
        out[rank] = (p.own, S.numpy()[:, p.own_local].copy(), len(p.cells))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("workload,world", [("config3s", 2), ("config2s", 3)])
def test_split_step_equals_single_rank(workload, world, oracle_lib):
    F, S0, dt, kw = _case(workload)
    ref = _advance(F.geometry(), S0, dt, kw, STEPS)
    with mp.Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_rank, args=(world, _free_port(), workload, out), nprocs=world, join=True)
        got = np.empty_like(ref)
        held = 0
        for r in range(world):
            (a, b), own, n = out[r]
            got[:, a:b] = own
            held += n
    assert np.array_equal(got, ref)
    assert held > F.n  # the halos overlap the neighbours' ranges


def test_ranges_and_halo():
    from forestfv_public_gb300 import partition as P
    rg = P.ranges(10, 3)
    assert rg[0][0] == 0 and rg[-1][1] == 10 and all(r[1] == s[0] for r, s in zip(rg, rg[1:]))
    assert max(b - a for a, b in rg) - min(b - a for a, b in rg) <= 1
    rg = P.ranges(1000, 4, weights=np.r_[np.ones(500), 3 * np.ones(500)])
    assert rg[0][0] == 0 and rg[-1][1] == 1000 and all(r[1] == s[0] for r, s in zip(rg, rg[1:]))
    F, _, _, _ = _case("config3s")
    geo = F.geometry()
    plans = P.plan(geo, 2, 2)
    for p in plans:
        assert np.array_equal(p.cells[p.own_local], np.arange(*p.own))
        for q, pos in p.recv.items():  # what q sends is what p receives, cell for cell
            assert np.array_equal(plans[q].cells[plans[q].send[p.rank]], p.cells[pos])
