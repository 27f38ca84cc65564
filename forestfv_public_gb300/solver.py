"""Host-side mirror of the reference's per-stage interface, over the C ABI.

  Solver.rk(irk, dt)            RK(irk, run) / m5_RK (RK.c:3-53), preceded for irk >= 1
                                by grad_scheme (grad_scheme.c:3-41) and RHS (RHS.c:3-72)
  Solver.advancetimeexplicit(dt) one step of RK_STEPS stages (advancetimeexplicit.c:3-28)
  Solver.step(dt, n)            n steps, each one CUDA graph launch
  Solver.cfl_dt(cfl)            CFL time step (the reference has a fixed DT)

State is structure-of-arrays, S[v, c], in the mesh's cell order.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .mesh import Mesh


def level_max(params) -> int:
    """The reference's LEVEL: the largest level any criterion names (inputset.c:106)."""
    return max(params.lvl_uniform, params.lvl_prs, params.lvl_rho, params.lvl_vel,
               params.lvl_inter0, params.lvl_inter1)


def adapt_changes(mesh: Mesh, split: np.ndarray) -> tuple[int, int]:
    """(leaves that split, sibling groups that merge) in a refineh pass with targets
    `split` (ffv_adapt_changes, host)."""
    split = np.ascontiguousarray(split, dtype=np.int32)
    ns, nm = ctypes.c_int64(), ctypes.c_int64()
    _lib.check(_lib.lib().ffv_adapt_changes(mesh.handle, split.ctypes.data, ctypes.byref(ns),
                                            ctypes.byref(nm)), "ffv_adapt_changes")
    return int(ns.value), int(nm.value)


def mesh_adapt(mesh: Mesh, split: np.ndarray):
    """The leaves and face tables of one refineh pass with targets `split` (host only,
    ffv_mesh_adapt); returns (Mesh, src) with every new leaf's source."""
    split = np.ascontiguousarray(split, dtype=np.int32)
    ns, nm = adapt_changes(mesh, split)
    src = np.empty(mesh.n + 7 * (ns - nm), np.int64)
    h = ctypes.c_void_p()
    _lib.check(_lib.lib().ffv_mesh_adapt(mesh.handle, split.ctypes.data, ctypes.byref(h),
                                         src.ctypes.data), "ffv_mesh_adapt")
    new = Mesh.from_handle(h, mesh.ntrees, mesh.bc, mesh.tree_edge)
    assert src.shape[0] == new.n
    return new, src


def would_change(mesh: Mesh, split: np.ndarray) -> bool:
    """Whether a refineh pass with targets `split` changes any leaf: a leaf wants a finer
    level, or eight sibling leaves all want a coarser one (refineh.c:10-57)."""
    ns, nm = adapt_changes(mesh, split)
    return ns + nm > 0


def tags_smooth(mesh: Mesh, lmax: int, split: np.ndarray) -> np.ndarray:
    """criterionsmth (ffv_tags_smooth) on a copy of the target levels `split`."""
    out = np.ascontiguousarray(split, dtype=np.int32).copy()
    _lib.check(_lib.lib().ffv_tags_smooth(mesh.handle, int(lmax), out.ctypes.data),
               "ffv_tags_smooth")
    return out


class Solver:
    def __init__(self, model: int = 0, order: int = 2, rk_steps: int = 2, gamma=(1.4,),
                 pinf=(0.0,), precision: int = _lib.FFV_FP64, device: int = 0, mu=None,
                 amin: float = 1e-6, avf_lim: float = 0.5, prelax: int = 3, zerou=(0, 0, 0),
                 flux_form: int = _lib.FFV_FLUX_REFERENCE, yield_stress=None):
        """model 0: gamma/pinf of the one material.  model 5: per-material gamma, pinf and
        mu (shear modulus, 0 for fluids), AMIN, AVF_LIM, PRELAX (1 or 3), ZEROU masks, and
        the flux form: FFV_FLUX_REFERENCE (the reference's m5 flux as written) or
        FFV_FLUX_CONSISTENT (its star-state energy, momentum-flux sign and deformation-flux
        sign made consistent with the rest of its HLLC solver; a deviation, see
        include/ffv.h); yield_stress: von Mises yield stress per material (0 or None: a
        hyperelastic solid, as the reference), a J2 radial return after each relaxation."""
        L = _lib.lib()
        p = _lib.Params()
        p.model, p.nmaterials, p.order, p.rk_steps, p.precision = model, len(gamma), order, rk_steps, precision
        p.prelax = prelax
        for i, g in enumerate(gamma):
            p.gamma[i] = g
        for i, q in enumerate(pinf):
            p.pinf[i] = q
        for i, q in enumerate(mu or ()):
            p.mu[i] = q
        p.amin, p.avf_lim = amin, avf_lim
        p.zerou[:] = tuple(zerou)
        p.flux_form = flux_form
        for i, y in enumerate(yield_stress or ()):
            p.yield_[i] = y
        self.params = p
        self.neq = 5 if model == 0 else 3 * len(gamma) + 12
        h = ctypes.c_void_p()
        _lib.check(L.ffv_create(ctypes.byref(h), ctypes.byref(p), device), "ffv_create")
        self._h = h
        self.device = device
        self.mesh: Mesh | None = None

    def set_mesh(self, mesh: Mesh) -> None:
        _lib.check(_lib.lib().ffv_set_mesh(self._h, mesh.handle), "ffv_set_mesh")
        self.mesh = mesh

    def upload_state(self, S: np.ndarray) -> None:
        S = np.ascontiguousarray(S, dtype=np.float64)
        assert S.shape == (self.neq, self.mesh.n), S.shape
        _lib.check(_lib.lib().ffv_upload_state(self._h, S.ctypes.data, self.mesh.n, self.neq),
                   "ffv_upload_state")

    def download_state(self, out: np.ndarray | None = None) -> np.ndarray:
        """The state [neq, n]; into `out` when given (a pinned host buffer copies at the
        link's full rate, a fresh pageable array goes through the driver's staging)."""
        if out is None:
            out = np.empty((self.neq, self.mesh.n))
        assert out.shape == (self.neq, self.mesh.n) and out.dtype == np.float64
        assert out.flags["C_CONTIGUOUS"]
        _lib.check(_lib.lib().ffv_download_state(self._h, out.ctypes.data, self.mesh.n, self.neq),
                   "ffv_download_state")
        return out

    def rk(self, irk: int, dt: float) -> None:
        _lib.check(_lib.lib().ffv_stage(self._h, irk, dt), "ffv_stage")

    def sync(self) -> None:
        _lib.check(_lib.lib().ffv_sync(self._h), "ffv_sync")

    def advancetimeexplicit(self, dt: float) -> None:
        self.step(dt, 1)

    def step(self, dt: float, nsteps: int = 1) -> None:
        _lib.check(_lib.lib().ffv_step(self._h, dt, nsteps), "ffv_step")

    def step_async(self, dt: float, nsteps: int = 1) -> None:
        _lib.check(_lib.lib().ffv_step_async(self._h, dt, nsteps), "ffv_step_async")

    def tags(self, params, with_raw: bool = False):
        """Refinement tags of the current state (ffv_tags): the smoothed target level per
        cell; with_raw also returns the level before smoothing and the interface layers
        SI [2, n].  params: a TagParams or the reference's 17 criterion inputs."""
        if not isinstance(params, _lib.TagParams):
            params = _lib.TagParams.from_tuple(params)
        n = self.mesh.n
        split = np.empty(n, np.int32)
        raw = np.empty(n, np.int32) if with_raw else None
        si = np.empty((2, n), np.int32) if with_raw else None
        _lib.check(_lib.lib().ffv_tags(self._h, self.mesh.handle, ctypes.byref(params),
                                       split.ctypes.data,
                                       raw.ctypes.data if with_raw else None,
                                       si.ctypes.data if with_raw else None), "ffv_tags")
        return (split, raw, si) if with_raw else split

    def tags_raw(self, params) -> np.ndarray:
        """The criterion's target level per cell before smoothing (ffv_tags_raw)."""
        if not isinstance(params, _lib.TagParams):
            params = _lib.TagParams.from_tuple(params)
        split = np.empty(self.mesh.n, np.int32)
        _lib.check(_lib.lib().ffv_tags_raw(self._h, self.mesh.handle, ctypes.byref(params),
                                           split.ctypes.data, None), "ffv_tags_raw")
        return split

    def tags_missed(self, params) -> int:
        """Number of cells whose raw target level is above their level (ffv_tags_missed):
        the plain criterion as a judge, counted on the device."""
        if not isinstance(params, _lib.TagParams):
            params = _lib.TagParams.from_tuple(params)
        out = ctypes.c_int64()
        _lib.check(_lib.lib().ffv_tags_missed(self._h, self.mesh.handle, ctypes.byref(params),
                                              ctypes.byref(out)), "ffv_tags_missed")
        return int(out.value)

    def adapt(self, split, with_src: bool = False, changes: tuple[int, int] | None = None):
        """One refineh pass (ffv_adapt) with target levels `split`; the solver continues on
        the returned mesh with the carried-over state.  with_src also returns every new
        leaf's source (ffv_adapt_map: the old leaf it copies, or -1 - j for a parent merged
        from old leaves j..j+7); `changes`, when the caller has them, are adapt_changes of
        `split` (they size the source array)."""
        split = np.ascontiguousarray(split, dtype=np.int32)
        assert split.shape == (self.mesh.n,)
        h = ctypes.c_void_p()
        src = None
        if with_src:
            ns, nm = changes if changes is not None else adapt_changes(self.mesh, split)
            src = np.empty(self.mesh.n + 7 * (ns - nm), np.int64)
        _lib.check(_lib.lib().ffv_adapt_map(self._h, self.mesh.handle, split.ctypes.data,
                                            ctypes.byref(h),
                                            src.ctypes.data if with_src else None), "ffv_adapt")
        old = self.mesh
        self.mesh = Mesh.from_handle(h, old.ntrees, old.bc, old.tree_edge)
        if with_src:
            assert src.shape[0] == self.mesh.n
            return self.mesh, src
        return self.mesh

    def meshadaptation(self, params) -> Mesh:
        """The reference's meshadaptation (meshadaptation.c:3-46): LEVEL + 1 rounds of the
        refinement tags and one refineh pass, LEVEL the largest level the criteria name."""
        if not isinstance(params, _lib.TagParams):
            params = _lib.TagParams.from_tuple(params)
        for _ in range(level_max(params) + 1):
            split = self.tags(params)
            if not would_change(self.mesh, split):
                break  # every further round sees the same state and mesh
            self.adapt(split)
        return self.mesh

    def conservation_sums(self) -> np.ndarray:
        """sum over cells of |V| S[v] per conserved variable, FP64 on the device
        (ffv_conservation_sums)."""
        out = np.empty(self.neq)
        _lib.check(_lib.lib().ffv_conservation_sums(self._h, out.ctypes.data),
                   "ffv_conservation_sums")
        return out

    def cfl_dt(self, cfl: float) -> float:
        out = ctypes.c_double()
        _lib.check(_lib.lib().ffv_cfl_dt(self._h, cfl, ctypes.byref(out)), "ffv_cfl_dt")
        return out.value

    def launches_per_step(self) -> int:
        n = ctypes.c_int32()
        _lib.check(_lib.lib().ffv_launches_per_step(self._h, ctypes.byref(n)), "ffv_launches_per_step")
        return n.value

    def profile_stage(self, irk: int, dt: float) -> dict:
        """Per-kernel durations (ms) of one stage, CUDA events on the solver's stream."""
        ms = np.zeros(16, dtype=np.float32)
        nk = ctypes.c_int32()
        L = _lib.lib()
        _lib.check(L.ffv_profile_stage(self._h, irk, dt, ms.ctypes.data, 16, ctypes.byref(nk)),
                   "ffv_profile_stage")
        out = {}
        for i in range(nk.value):
            name = L.ffv_stage_kernel_name(self._h, i).decode()
            out[name] = out.get(name, 0.0) + float(ms[i])
        return out

    def stream_handle(self) -> int:
        p = ctypes.c_void_p()
        _lib.check(_lib.lib().ffv_stream(self._h, ctypes.byref(p)), "ffv_stream")
        return p.value

    def device_state_ptr(self) -> int:
        p = ctypes.c_void_p()
        _lib.check(_lib.lib().ffv_state_device_ptr(self._h, ctypes.byref(p)), "ffv_state_device_ptr")
        return p.value

    def close(self) -> None:
        if getattr(self, "_h", None):
            _lib.lib().ffv_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
