"""The time loop with mesh adaptation, plain and learned.

Plain AMR is the reference's loop (loop.c:13-30): before step s (counted from 0) with
(s + 1) % every == 0 it runs meshadaptation (meshadaptation.c:3-46), LEVEL + 1 rounds of
the refinement tags and one refineh pass.  A round that would change no leaf ends the
rounds early: every further round would see the same state and mesh, so the result is
the reference's.

Learned AMR (no counterpart in the reference) regrids less often.  The network of
indicator.py runs every `infer_every` steps and marks the cells whose probability of being
flagged by the criterion `horizon` steps ahead exceeds `threshold`; the marks accumulate
until the next regrid.  At the steps where plain AMR would regrid, the plain criterion
runs as a judge on the device (ffv_tags_missed): when no cell is below its target level
the regrid is skipped, otherwise -- and after `max_skips` skipped regrids in a row, so that
the mesh can coarsen -- a regrid runs.  Its target is the criterion's raw level, raised on
the marked cells to the level the gradient criteria assign (`pre_level`), then smoothed
(criterionsmth); later rounds carry the marks to the new leaves (children inherit them), and
the rounds end as soon as every leaf has reached the round's target (what the criterion
wants on the new state, the next judge finds).  Any cell the
criterion flags is refined whether or not the network marked it: the criterion is the
fallback.
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from .solver import Solver, adapt_changes, level_max, tags_smooth, would_change


@dataclass
class AMRStats:
    steps: int = 0
    cell_updates: int = 0
    regrids: int = 0
    rounds: int = 0
    judged: int = 0
    skipped: int = 0
    missed: list = field(default_factory=list)
    cells: list = field(default_factory=list)
    t_step: float = 0.0
    t_regrid: float = 0.0
    t_judge: float = 0.0
    t_infer: float = 0.0
    inferences: int = 0

    @property
    def seconds(self) -> float:
        return self.t_step + self.t_regrid + self.t_judge + self.t_infer

    def as_dict(self) -> dict:
        return {"steps": self.steps, "cell_updates": self.cell_updates,
                "regrids": self.regrids, "rounds": self.rounds, "judged": self.judged,
                "skipped": self.skipped, "missed": self.missed,
                "cells_min": int(min(self.cells)) if self.cells else 0,
                "cells_max": int(max(self.cells)) if self.cells else 0,
                "seconds": self.seconds, "step_s": self.t_step, "regrid_s": self.t_regrid,
                "judge_s": self.t_judge, "infer_s": self.t_infer, "inferences": self.inferences,
                "cell_updates_per_s": self.cell_updates / max(self.seconds, 1e-30)}


def carry_marks(src: np.ndarray, marks: np.ndarray) -> np.ndarray:
    """Marks of the old leaves carried to the new leaves of a refineh pass, given every new
    leaf's source (ffv_adapt_map): a kept leaf or a child keeps its (parent's) mark, a
    merged parent takes any of its eight children's."""
    out = np.empty(src.shape[0], bool)
    keep = src >= 0
    out[keep] = marks[src[keep]]
    j = -1 - src[~keep]
    acc = np.zeros(j.shape[0], bool)
    for q in range(8):
        acc |= marks[j + q]
    out[~keep] = acc
    return out


def gradient_level(params) -> int:
    """The level the gradient criteria assign to a flagged cell (the largest of the
    enabled ones; LEVEL when none is enabled)."""
    lv = [l for on, l in ((params.grad_prs, params.lvl_prs), (params.grad_rho, params.lvl_rho),
                          (params.grad_vel, params.lvl_vel)) if on == 1]
    return max(lv) if lv else level_max(params)


class AdaptiveRun:
    def __init__(self, solver: Solver, tag_params, every: int = 8, indicator=None,
                 threshold: float = 0.5, infer_every: int = 1, max_skips: int = 3,
                 pre_level: int | None = None):
        if not isinstance(tag_params, _lib.TagParams):
            tag_params = _lib.TagParams.from_tuple(tag_params)
        self.solver = solver
        self.params = tag_params
        self.every = int(every)
        self.indicator = indicator
        self.threshold = float(threshold)
        self.infer_every = max(1, int(infer_every))
        self.max_skips = int(max_skips)
        self.lmax = level_max(tag_params)
        self.pre_level = gradient_level(tag_params) if pre_level is None else int(pre_level)
        self.marks: np.ndarray | None = None
        self._skips = 0
        self.stats = AMRStats()

    # ------------------------------------------------------------------ regrids
    def meshadaptation(self) -> int:
        """The reference's meshadaptation with the early end; returns the rounds run."""
        s, rounds = self.solver, 0
        for _ in range(self.lmax + 1):
            split = s.tags(self.params)
            if not would_change(s.mesh, split):
                break
            s.adapt(split)
            rounds += 1
        return rounds

    def _mark(self, accumulate: bool) -> None:
        """Run the network and OR its marks into the device buffer (no copy back)."""
        import torch
        n = self.solver.mesh.n
        if self.marks is None or self.marks.shape[0] != n:
            # no fill: the first mark overwrites every entry (and a fill on torch's stream
            # would race with the mark kernel on the solver's)
            self.marks = torch.empty(n, dtype=torch.uint8, device=f"cuda:{self.indicator.device}")
            accumulate = False
        self.indicator.mark(self.solver, self.threshold, self.marks, accumulate)

    def learned_regrid(self) -> int:
        """A regrid whose target is the criterion's, raised to pre_level on marked cells."""
        s, rounds = self.solver, 0
        if self.marks is None or self.marks.shape[0] != s.mesh.n:
            self._mark(accumulate=False)
        s.sync()
        marks = self.marks.cpu().numpy().astype(bool)
        for _ in range(self.lmax + 1):
            tgt = s.tags_raw(self.params)
            np.maximum(tgt, self.pre_level, out=tgt, where=marks)
            tgt = tags_smooth(s.mesh, self.lmax, tgt)
            changes = adapt_changes(s.mesh, tgt)
            if changes[0] + changes[1] == 0:
                break
            level = s.mesh.level
            _, src = s.adapt(tgt, with_src=True, changes=changes)
            rounds += 1
            # every leaf at (or, for a sibling group that could not merge, above) its
            # target: no further round, whatever the criterion wants on the new state the
            # next judge finds.  A leaf splits exactly when its target is above its level
            # (refineh.c:10-57), into children one level finer, and a kept leaf's target is
            # not above its level: a new leaf from an old one is below its target only where
            # the old leaf's target was two or more levels above it.
            if not np.any(tgt > level + 1):
                break
            marks = carry_marks(src, marks)
        self.marks = None
        return rounds

    # ------------------------------------------------------------------ the loop
    def run(self, dt: float, nsteps: int) -> AMRStats:
        s, st = self.solver, self.stats
        for _ in range(nsteps):
            k = st.steps
            if (k + 1) % self.every == 0:
                if self.indicator is None:
                    t0 = time.perf_counter()
                    st.rounds += self.meshadaptation()
                    st.regrids += 1
                    st.t_regrid += time.perf_counter() - t0
                else:
                    t0 = time.perf_counter()
                    missed = s.tags_missed(self.params)
                    st.judged += 1
                    st.missed.append(missed)
                    st.t_judge += time.perf_counter() - t0
                    if missed > 0 or self._skips >= self.max_skips:
                        t0 = time.perf_counter()
                        st.rounds += self.learned_regrid()
                        st.regrids += 1
                        self._skips = 0
                        st.t_regrid += time.perf_counter() - t0
                    else:
                        self._skips += 1
                        st.skipped += 1
            if self.indicator is not None and k % self.infer_every == 0:
                t0 = time.perf_counter()
                self._mark(accumulate=True)
                st.inferences += 1
                st.t_infer += time.perf_counter() - t0
            t0 = time.perf_counter()
            s.step(dt, 1)
            st.t_step += time.perf_counter() - t0
            st.steps += 1
            st.cell_updates += s.mesh.n
            st.cells.append(s.mesh.n)
        return st
