"""Learned refinement indicator (host side): the network of csrc/ffv_mlp.cu behind
ffv_mlp_*, the collection of training pairs from the solver's own runs and the decision
rule that combines it with the plain criterion.

Training pairs: the feature rows of a state at step n and the label "the plain criterion
(ffv_tags) asks for a finer level than the cell has, at step n + horizon".  The network is
evaluated every step; the plain criterion every `judge_every` steps as judge and fallback:
a cell is marked when the network's probability exceeds the threshold or the criterion
asks for refinement (any cell the criterion flags and the network missed is refined)."""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib

NPARAM = 12929
KIN = 144


class Indicator:
    def __init__(self, device: int = 0, seed: int = 1):
        h = ctypes.c_void_p()
        _lib.check(_lib.lib().ffv_mlp_create(ctypes.byref(h), device, seed), "ffv_mlp_create")
        self._h = h
        self.device = device
        self.mean = np.zeros(5, np.float32)
        self.std = np.ones(5, np.float32)

    def close(self) -> None:
        if self._h:
            _lib.lib().ffv_mlp_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # parameters -------------------------------------------------------------------
    def params(self) -> np.ndarray:
        P = np.empty(NPARAM, np.float32)
        _lib.check(_lib.lib().ffv_mlp_get_params(self._h, P.ctypes.data), "ffv_mlp_get_params")
        return P

    def set_params(self, P) -> None:
        P = np.ascontiguousarray(P, dtype=np.float32)
        assert P.shape == (NPARAM,)
        _lib.check(_lib.lib().ffv_mlp_set_params(self._h, P.ctypes.data), "ffv_mlp_set_params")

    def set_norm(self, mean, std) -> None:
        self.mean = np.ascontiguousarray(mean, dtype=np.float32)
        self.std = np.ascontiguousarray(std, dtype=np.float32)
        _lib.check(_lib.lib().ffv_mlp_set_norm(self._h, self.mean.ctypes.data,
                                               self.std.ctypes.data), "ffv_mlp_set_norm")

    # device data (torch tensors as plain device buffers) ------------------------
    def fields(self, solver):
        import torch
        F = torch.empty((5, solver.mesh.n), dtype=torch.float32, device=f"cuda:{self.device}")
        _lib.check(_lib.lib().ffv_mlp_fields(solver._h, F.data_ptr()), "ffv_mlp_fields")
        return F

    def features(self, solver):
        import torch
        X = torch.empty((solver.mesh.n, KIN), dtype=torch.bfloat16, device=f"cuda:{self.device}")
        _lib.check(_lib.lib().ffv_mlp_features(solver._h, self._h, X.data_ptr()),
                   "ffv_mlp_features")
        return X

    def forward(self, X):
        import torch
        p = torch.empty(X.shape[0], dtype=torch.float32, device=X.device)
        _lib.check(_lib.lib().ffv_mlp_forward(self._h, X.data_ptr(), X.shape[0], p.data_ptr()),
                   "ffv_mlp_forward")
        return p

    def predict(self, solver) -> np.ndarray:
        p = np.empty(solver.mesh.n, np.float32)
        _lib.check(_lib.lib().ffv_mlp_predict(solver._h, self._h, p.ctypes.data),
                   "ffv_mlp_predict")
        return p

    def mark(self, solver, threshold: float, marks, accumulate: bool) -> None:
        """marks (device uint8 tensor [n]) |= probability > threshold, on the solver's
        stream, nothing copied back (ffv_mlp_mark)."""
        _lib.check(_lib.lib().ffv_mlp_mark(solver._h, self._h, float(threshold),
                                           marks.data_ptr(), 1 if accumulate else 0),
                   "ffv_mlp_mark")

    def grad(self, X, y, B: int | None = None):
        B = X.shape[0] if B is None else B
        g = np.empty(NPARAM, np.float32)
        loss = ctypes.c_float()
        _lib.check(_lib.lib().ffv_mlp_grad(self._h, X.data_ptr(), y.data_ptr(), B, g.ctypes.data,
                                           ctypes.byref(loss)), "ffv_mlp_grad")
        return g, float(loss.value)

    def train(self, X, y, steps: int, batch: int = 8192, lr: float = 1e-3, wd: float = 1e-4,
              seed: int = 1, record_loss: bool = True) -> np.ndarray:
        losses = np.zeros(steps, np.float32)
        _lib.check(_lib.lib().ffv_mlp_train(self._h, X.data_ptr(), y.data_ptr(), X.shape[0],
                                            batch, steps, lr, wd, seed,
                                            losses.ctypes.data if record_loss else None),
                   "ffv_mlp_train")
        return losses


def field_norm(F_list) -> tuple[np.ndarray, np.ndarray]:
    """Per-field mean and standard deviation over snapshots of fields [5, n] (host)."""
    cat = np.concatenate([np.asarray(F) for F in F_list], axis=1)
    mean = cat.mean(axis=1)
    std = np.maximum(cat.std(axis=1), 1e-6)
    return mean.astype(np.float32), std.astype(np.float32)


def needs_refinement(split: np.ndarray, level: np.ndarray) -> np.ndarray:
    """The label: the criterion's target level is above the cell's level."""
    return split > level


def collect(solver, indicator: Indicator, tag_params, dt: float, snapshots: int, every: int,
            horizon: int):
    """Run the solver and gather (features at step n, label at step n + horizon) pairs from
    `snapshots` states `every` steps apart.  Returns device tensors X [N, 144] (BF16) and
    y [N] (FP32) and the host criterion tags at every snapshot step (for evaluation)."""
    import torch
    level = solver.mesh.level
    Xs, ys, tags_now, tags_future = [], [], [], []
    for _ in range(snapshots):
        Xs.append(indicator.features(solver))
        tags_now.append(solver.tags(tag_params))
        solver.step(dt, horizon)
        fut = solver.tags(tag_params)
        tags_future.append(fut)
        ys.append(torch.from_numpy(needs_refinement(fut, level).astype(np.float32)))
        if every > horizon:
            solver.step(dt, every - horizon)
    X = torch.cat(Xs)
    y = torch.cat(ys).to(X.device)
    return X, y, tags_now, tags_future


def collect_window(solver, indicator: Indicator, tag_params, dt: float, horizon: int):
    """One training snapshot for pre-refinement: the feature rows of the current state and
    the label "the plain criterion asks for a finer level than the cell has at some step
    of the next `horizon`" (raw criterion levels, ffv_tags_raw, one per step).  Advances the
    solver `horizon` steps on its current mesh.  Returns device X [n, 144] and y [n]."""
    import torch
    level = solver.mesh.level
    X = indicator.features(solver)
    hit = np.zeros(solver.mesh.n, bool)
    for _ in range(horizon):
        solver.step(dt, 1)
        hit |= solver.tags_raw(tag_params) > level
    return X, torch.from_numpy(hit.astype(np.float32)).to(X.device)


def coverage(flag_now: np.ndarray, flag_future: np.ndarray) -> tuple[float, int]:
    """Fraction of the cells flagged at the future step that are flagged now, and the number
    of cells flagged now."""
    fut = flag_future.astype(bool)
    return float((flag_now & fut).sum() / max(fut.sum(), 1)), int(flag_now.sum())


def gain_report(indicator: Indicator, solver, tag_params, dt: float, snapshots: int, every: int,
                horizon: int, threshold: float = 0.5) -> dict:
    """On a run the network was not trained on: how many of the cells that the plain
    criterion will flag `horizon` steps later are already marked at step n, by the
    criterion alone and by the criterion together with the network."""
    level = solver.mesh.level
    cov_c, cov_u, n_c, n_u = [], [], 0, 0
    for _ in range(snapshots):
        now = needs_refinement(solver.tags(tag_params), level)
        pred = indicator.predict(solver) > threshold
        solver.step(dt, horizon)
        fut = needs_refinement(solver.tags(tag_params), level)
        a, na = coverage(now, fut)
        b, nb = coverage(now | pred, fut)
        cov_c.append(a)
        cov_u.append(b)
        n_c += na
        n_u += nb
        if every > horizon:
            solver.step(dt, every - horizon)
    return {"coverage_criterion": float(np.mean(cov_c)),
            "coverage_criterion_and_network": float(np.mean(cov_u)),
            "cells_marked_criterion": n_c, "cells_marked_criterion_and_network": n_u}
