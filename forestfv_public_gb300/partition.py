"""The step split over several GPUs: contiguous Morton ranges of the leaves, one per rank.

The reference partitions its trees with METIS / ParMETIS (partitiondrys.c:61,
repartition_parmetis.c:267), gives each rank proxy copies of its neighbours' leaves
(rebuildprox.c:3-246) and exchanges their states and face states with MPI after every stage
(communicate.c:45-248, communicate_nb_S.c:3-130, advancetimeexplicit.c:23).  Here:

* Partition: the leaf list (a global Morton order) cut into `nranks` contiguous ranges of
  equal weight (cells, or a cost per cell).
* Halo: each rank holds its own cells and every cell within `depth` face hops of them, as a
  mesh of its own (ffv_mesh_build_part: faces towards cells it does not hold are transmissive
  boundaries).  A stage reads neighbours two hops out (a face state from the neighbour's
  neighbours, the flux from both face states) and the ghost-fluid fixes one more, so a halo of
  3 x rk_steps hops keeps the rank's own cells exact through a whole time step
  (HALO_HOPS_PER_STAGE); the rank advances its whole part, one CUDA graph per step, and the
  halo's outer layers go stale.
* Exchange: one per time step, after it: every rank sends the states of its own cells that
  other ranks hold as halo and receives those of its halo cells, packed into one buffer per
  rank pair (torch.distributed point-to-point: NCCL between GPUs, gloo on the CPU).  Global
  reductions (the CFL dt, the conservation sums) are all-reduces of one or a few doubles.

A rank's leaves keep their relative order, so the reference's order-dependent walks (flux
reuse from the earlier leaf, the ghost-fluid fixes reading earlier neighbours updated and
later ones not) see the same order on every rank as on one: the rank's own cells come out
bit-identical to the single-GPU step (tests/test_partition.py, tests/test_gpu_partition.py).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

HALO_HOPS_PER_STAGE = 3


def ranges(n: int, nranks: int, weights=None) -> list[tuple[int, int]]:
    """Contiguous ranges [a, b) of the n leaves, one per rank, of equal total weight."""
    w = np.ones(n) if weights is None else np.asarray(weights, np.float64)
    cum = np.concatenate([[0.0], np.cumsum(w)])
    cuts = [0]
    for r in range(1, nranks):
        cuts.append(int(np.searchsorted(cum, cum[-1] * r / nranks)))
    cuts.append(n)
    return [(cuts[r], cuts[r + 1]) for r in range(nranks)]


def adjacency(geo: dict) -> tuple[np.ndarray, np.ndarray]:
    """Face neighbours of every cell (all sub-neighbours of a face with four finer ones) as a
    CSR pair (indptr, indices), from the reference-form geometry (Mesh.export())."""
    nb = np.asarray(geo["nb"]).reshape(len(geo["vol"]), 24)
    valid = nb >= 0
    indptr = np.concatenate([[0], np.cumsum(valid.sum(axis=1))]).astype(np.int64)
    return indptr, nb[valid].astype(np.int64)


def closure(indptr: np.ndarray, indices: np.ndarray, cells: np.ndarray, hops: int) -> np.ndarray:
    """The cells within `hops` face hops of `cells` (those included), sorted."""
    n = len(indptr) - 1
    inside = np.zeros(n, bool)
    inside[cells] = True
    frontier = np.asarray(cells, np.int64)
    for _ in range(hops):
        if len(frontier) == 0:
            break
        starts, ends = indptr[frontier], indptr[frontier + 1]
        lens = ends - starts
        idx = np.repeat(starts - np.concatenate([[0], np.cumsum(lens)[:-1]]), lens) + np.arange(lens.sum())
        nbrs = np.unique(indices[idx])
        frontier = nbrs[~inside[nbrs]]
        inside[frontier] = True
    return np.flatnonzero(inside)


@dataclass
class RankPlan:
    """One rank's part: its own range, the cells it holds (own and halo, global indices in
    leaf order), where its own cells sit among them, and the exchange lists."""
    rank: int
    nranks: int
    own: tuple[int, int]
    cells: np.ndarray                   # global indices held, sorted
    own_local: np.ndarray               # positions of the own cells within `cells`
    send: dict = field(default_factory=dict)   # peer -> positions (in `cells`) to send
    recv: dict = field(default_factory=dict)   # peer -> positions (in `cells`) to receive

    @property
    def n(self) -> int:
        return len(self.cells)


def plan(geo: dict, nranks: int, hops: int, weights=None) -> list[RankPlan]:
    """Partition and halo plans of all ranks (every rank computes the same plans)."""
    n = len(geo["vol"])
    indptr, indices = adjacency(geo)
    rg = ranges(n, nranks, weights)
    owner = np.zeros(n, np.int32)
    for r, (a, b) in enumerate(rg):
        owner[a:b] = r
    plans = []
    for r, (a, b) in enumerate(rg):
        cells = closure(indptr, indices, np.arange(a, b), hops)
        own_local = np.flatnonzero((cells >= a) & (cells < b))
        plans.append(RankPlan(r, nranks, (a, b), cells, own_local))
    for p in plans:
        halo = np.flatnonzero((p.cells < p.own[0]) | (p.cells >= p.own[1]))
        for q in np.unique(owner[p.cells[halo]]):
            q = int(q)
            mine = halo[owner[p.cells[halo]] == q]         # my halo cells owned by q
            p.recv[q] = mine
            src = plans[q]
            plans[q].send[p.rank] = np.searchsorted(src.cells, p.cells[mine])
    return plans


def exchange(S, p: RankPlan, group=None) -> None:
    """The halo exchange of one rank, in place on its state S (a torch tensor [neq, p.n] on
    the rank's device): its own cells that peers hold go out, its halo cells come in, one
    packed buffer per peer and direction."""
    import torch
    import torch.distributed as dist
    reqs, inbox = [], []
    for q, pos in sorted(p.send.items()):
        buf = S[:, torch.as_tensor(pos, device=S.device)].contiguous()
        reqs.append(dist.isend(buf, q, group=group))
        inbox.append(buf)  # keep alive until sent
    recvd = []
    for q, pos in sorted(p.recv.items()):
        buf = torch.empty((S.shape[0], len(pos)), dtype=S.dtype, device=S.device)
        reqs.append(dist.irecv(buf, q, group=group))
        recvd.append((pos, buf))
    for r in reqs:
        r.wait()
    for pos, buf in recvd:
        S[:, torch.as_tensor(pos, device=S.device)] = buf


class _DeviceArray:
    """__cuda_array_interface__ of the solver's state (a view, no copy)."""

    def __init__(self, ptr: int, neq: int, n: int):
        self.__cuda_array_interface__ = {"shape": (neq, n), "typestr": "<f8",
                                         "data": (ptr, False), "version": 3, "strides": None}


class RankStep:
    """One rank of the split step on its GPU: a Solver on the rank's part of the forest and
    the halo exchange after every time step over torch.distributed (NCCL)."""

    def __init__(self, ntrees, leaves, bc, p: RankPlan, solver_kwargs: dict, device: int = 0,
                 group=None):
        from .mesh import Leaves, Mesh
        from .solver import Solver
        c = p.cells
        self.plan = p
        self.group = group
        self.mesh = Mesh(ntrees, Leaves(leaves.tree_ijk[c], leaves.level[c], leaves.cell_ijk[c]),
                         bc=bc, part=True)
        self.solver = Solver(device=device, **solver_kwargs)
        self.solver.set_mesh(self.mesh)

    def upload(self, S_global: np.ndarray) -> None:
        self.solver.upload_state(np.ascontiguousarray(S_global[:, self.plan.cells]))

    def state(self):
        """The solver's device state as a torch tensor [neq, n] (a view)."""
        import torch
        s = self.solver
        return torch.as_tensor(_DeviceArray(s.device_state_ptr(), s.neq, self.plan.n),
                               device=f"cuda:{s.device}")

    def step(self, dt: float, nsteps: int = 1) -> None:
        import torch
        for _ in range(nsteps):
            self.solver.step(dt, 1)  # synchronises the solver's stream
            exchange(self.state(), self.plan, self.group)
            torch.cuda.synchronize(self.solver.device)

    def own_state(self) -> np.ndarray:
        return self.solver.download_state()[:, self.plan.own_local]

    def close(self) -> None:
        self.solver.close()
        self.mesh.close()
