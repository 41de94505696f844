"""Host-side mirror of tetemoko's level/patch interfaces over the C ABI.

Names and argument meaning follow the reference:
  * LinElastPatchGodunov.update_state  -> LinElastPatchGodunov::updateState
    (srcLinElast/LinElastPatchGodunov.cpp:101-129) on device FABs;
  * LinElastPatchGodunov.plastic_update -> LinElastPhysics::plasticUpdate;
  * LinElastLevelGodunov.step / plastic_update -> LinElastLevelGodunov::step /
    plasticUpdate (srcLinElast/LinElastLevelGodunov.cpp:174-398, 643-667) on a
    device-resident level.
Device memory and streams come from PyTorch; every computation runs in the
CUDA library (libtetemoko_gb300.so) and fails loudly when it is missing.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _capi as A


def _torch():
    import torch
    return torch


def _stream_ptr(stream) -> int | None:
    if stream is None:
        torch = _torch()
        return torch.cuda.current_stream().cuda_stream
    return int(stream.cuda_stream) if hasattr(stream, "cuda_stream") else int(stream)


class Context:
    """Per-scenario parameters on the device (replaces the COMMON blocks)."""

    def __init__(self, sc):
        self.sc = sc
        self.lib = A.lib()
        h = C.c_void_p()
        rs = C.byref(sc.rs) if sc.rs is not None else None
        sw = C.byref(sc.sw) if sc.sw is not None else None
        pl = C.byref(sc.plastic) if sc.plastic is not None else None
        A.check(self.lib.tmk_context_create(C.byref(sc.elastic), C.byref(sc.scheme), rs, sw, pl, C.byref(h)),
                "tmk_context_create")
        self.h = h

    def constants(self) -> dict:
        out = (C.c_double * 5)()
        A.check(self.lib.tmk_context_constants(self.h, out), "tmk_context_constants")
        return dict(rho=out[0], lam=out[1], K=out[2], Zs=out[3], Zp=out[4])

    def close(self):
        if self.h:
            self.lib.tmk_context_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _fab(t, lo0, lo1) -> A.Fab:
    """tmk_fab over a (ncomp, ny, nx) float64 CUDA tensor whose cell (0,0) is (lo0, lo1)."""
    assert t.dtype == _torch().float64 and t.is_cuda and t.is_contiguous()
    f = A.Fab()
    f.data = t.data_ptr()
    f.lo[0], f.lo[1] = lo0, lo1
    f.hi[0], f.hi[1] = lo0 + t.shape[-1] - 1, lo1 + t.shape[-2] - 1
    f.ncomp = t.shape[0]
    return f


class LinElastPatchGodunov:
    """Patch integrator on caller-owned device FABs (FP64)."""

    def __init__(self, ctx: Context, domain=None, dx: float | None = None):
        self.ctx = ctx
        sc = ctx.sc
        self.domain = domain or (0, 0, sc.nx - 1, sc.ny - 1)
        self.dx = sc.dx if dx is None else dx
        self.time = 0.0
        self.box = None

    def set_current_time(self, t: float):
        self.time = t

    def set_current_box(self, box):
        self.box = tuple(box)

    def update_state(self, U, ulo, dt: float, B=None, bxlo: int = 0, with_flux: bool = False, stream=None):
        """Advance the valid box of U (ncomp=22, FP64 CUDA tensor whose first
        cell is `ulo`) by dt; B (fault row, cells from bxlo) updated in place.
        Returns (max_wave_speed, Fx, Fy)."""
        torch = _torch()
        v = A.box(*self.box)
        d = A.box(*self.domain)
        Uf = _fab(U, *ulo)
        Bf = None
        if B is not None:
            Bf = A.Fab()
            Bf.data = B.data_ptr()
            Bf.lo[0], Bf.lo[1] = bxlo, self.domain[1]
            Bf.hi[0], Bf.hi[1] = bxlo + B.shape[-1] - 1, self.domain[1]
            Bf.ncomp = B.shape[0]
        Fx = Fy = None
        Fxf = Fyf = None
        if with_flux:
            nx = self.box[2] - self.box[0] + 1
            ny = self.box[3] - self.box[1] + 1
            Fx = torch.empty((22, ny, nx + 1), dtype=torch.float64, device=U.device)
            Fy = torch.empty((22, ny + 1, nx), dtype=torch.float64, device=U.device)
            Fxf = _fab(Fx, self.box[0], self.box[1])
            Fyf = _fab(Fy, self.box[0], self.box[1])
        mws = C.c_double(0.0)
        A.check(self.ctx.lib.tmk_patch_update_state(
            self.ctx.h, C.byref(Uf), C.byref(Bf) if Bf is not None else None,
            C.byref(Fxf) if Fxf is not None else None, C.byref(Fyf) if Fyf is not None else None,
            C.byref(v), C.byref(d), self.dx, self.time, dt, C.byref(mws), _stream_ptr(stream)),
            "tmk_patch_update_state")
        return mws.value, Fx, Fy

    def plastic_update(self, U, ulo, dt: float, box=None, stream=None):
        b = A.box(*(box or self.box))
        A.check(self.ctx.lib.tmk_plastic_update(self.ctx.h, C.byref(_fab(U, *ulo)), C.byref(b), dt,
                                                _stream_ptr(stream)), "tmk_plastic_update")


def _fab3(t, lo) -> A.Fab3:
    """tmk_fab3 over a (ncomp, nz, ny, nx) float64 CUDA tensor whose first cell is lo = (i, j, k)."""
    assert t.dtype == _torch().float64 and t.is_cuda and t.is_contiguous() and t.dim() == 4
    f = A.Fab3()
    f.data = t.data_ptr()
    for d in range(3):
        f.lo[d] = lo[d]
        f.hi[d] = lo[d] + t.shape[3 - d] - 1
    f.ncomp = t.shape[0]
    return f


class LinElastPatchGodunov3D:
    """Patch integrator of a CH_SPACEDIM == 3 build (LinElastPatchGodunov with
    the 3-D corner transport upwind corrections) on caller-owned device FABs
    (FP64).  Boxes are ((lo0, lo1, lo2), (hi0, hi1, hi2)); the fault is the
    domain's y-lo plane."""

    def __init__(self, ctx: Context, domain, dx: float | None = None):
        self.ctx = ctx
        self.domain = (tuple(domain[0]), tuple(domain[1]))
        self.dx = ctx.sc.dx if dx is None else dx
        self.time = 0.0
        self.box = None

    def set_current_time(self, t: float):
        self.time = t

    def set_current_box(self, box):
        self.box = (tuple(box[0]), tuple(box[1]))

    def update_state(self, U, ulo, dt: float, B=None, blo=(0, 0), with_flux: bool = False, stream=None):
        """Advance the valid box of U ((22, nz, ny, nx) FP64 CUDA tensor whose
        first cell is ulo = (i, j, k)) by dt; B ((nb, nz_b, nx_b), first face
        blo = (i, k) on the fault plane) updated in place.  Returns
        (max_wave_speed, [F0, F1, F2])."""
        torch = _torch()
        v = A.box3(*self.box)
        d = A.box3(*self.domain)
        Uf = _fab3(U, ulo)
        Bf = None
        if B is not None:
            Bf = A.Fab3()
            Bf.data = B.data_ptr()
            Bf.lo[0], Bf.lo[1], Bf.lo[2] = blo[0], self.domain[0][1], blo[1]
            Bf.hi[0], Bf.hi[1], Bf.hi[2] = blo[0] + B.shape[2] - 1, self.domain[0][1], blo[1] + B.shape[1] - 1
            Bf.ncomp = B.shape[0]
        F = [None, None, None]
        Ff = [None, None, None]
        if with_flux:
            n = [self.box[1][e] - self.box[0][e] + 1 for e in range(3)]
            for e in range(3):
                m = list(n)
                m[e] += 1
                F[e] = torch.empty((22, m[2], m[1], m[0]), dtype=torch.float64, device=U.device)
                Ff[e] = _fab3(F[e], self.box[0])
        mws = C.c_double(0.0)
        ref = lambda x: C.byref(x) if x is not None else None
        A.check(self.ctx.lib.tmk_patch_update_state_3d(
            self.ctx.h, C.byref(Uf), ref(Bf), ref(Ff[0]), ref(Ff[1]), ref(Ff[2]), C.byref(v), C.byref(d),
            self.dx, self.time, dt, C.byref(mws), _stream_ptr(stream)), "tmk_patch_update_state_3d")
        return mws.value, F

    def update_states(self, patches, dt: float, stream=None):
        """The level's patch loop in one batched call: `patches` is a list of
        (valid box, U, ulo, B or None, blo); the patches' passes run as one
        launch each over all of them.  Returns the max wave speed."""
        n = len(patches)
        Ua = (A.Fab3 * n)()
        Ba = (A.Fab3 * n)()
        Va = (A.Box3 * n)()
        anyB = False
        for p, (valid, U, ulo, B, blo) in enumerate(patches):
            Ua[p] = _fab3(U, ulo)
            Va[p] = A.box3(*valid)
            if B is not None:
                anyB = True
                f = A.Fab3()
                f.data = B.data_ptr()
                f.lo[0], f.lo[1], f.lo[2] = blo[0], self.domain[0][1], blo[1]
                f.hi[0], f.hi[1], f.hi[2] = blo[0] + B.shape[2] - 1, self.domain[0][1], blo[1] + B.shape[1] - 1
                f.ncomp = B.shape[0]
                Ba[p] = f
        mws = C.c_double(0.0)
        d = A.box3(*self.domain)
        A.check(self.ctx.lib.tmk_patches_update_state_3d(
            self.ctx.h, n, Ua, Ba if anyB else None, None, None, None, Va, C.byref(d), self.dx, self.time, dt,
            C.byref(mws), _stream_ptr(stream)), "tmk_patches_update_state_3d")
        return mws.value

    def plastic_update(self, U, ulo, dt: float, box=None, stream=None):
        b = A.box3(*(box or self.box))
        A.check(self.ctx.lib.tmk_plastic_update_3d(self.ctx.h, C.byref(_fab3(U, ulo)), C.byref(b), dt,
                                                   _stream_ptr(stream)), "tmk_plastic_update_3d")


class LinElastLevelGodunov3D:
    """Device-resident level of a CH_SPACEDIM == 3 build (tmk_level3d): the
    level owns each patch's FP64 state FAB (22, nz+8, ny+8, nx+8) over the
    valid box grown by 4 ghosts and, on the fault plane, its fault data
    (nbdry, nz+8, nx+8); a step exchanges ghost cells on the device and runs
    the batched 3-D patch loop (and the plastic correction on plastic
    schemes).  Boxes are ((lo0, lo1, lo2), (hi0, hi1, hi2))."""

    def __init__(self, ctx: Context, boxes, domain, dx: float | None = None):
        self.ctx = ctx
        self.lib = ctx.lib
        self.boxes = [(tuple(b[0]), tuple(b[1])) for b in boxes]
        self.domain = (tuple(domain[0]), tuple(domain[1]))
        self.dx = ctx.sc.dx if dx is None else dx
        arr = (A.Box3 * len(self.boxes))(*[A.box3(*b) for b in self.boxes])
        h = C.c_void_p()
        A.check(self.lib.tmk_level3d_create(ctx.h, C.byref(A.box3(*self.domain)), self.dx, len(self.boxes), arr,
                                            C.byref(h)), "tmk_level3d_create")
        self.h = h

    def touches_fault(self, p) -> bool:
        return self.ctx.sc.scheme.fault_law != A.TMK_FAULT_NONE and self.boxes[p][0][1] == self.domain[0][1]

    def patch_shapes(self, p):
        (lo, hi), g = self.boxes[p], A.TMK_NGHOST
        n = [hi[d] - lo[d] + 1 + 2 * g for d in range(3)]
        return (22, n[2], n[1], n[0]), (self.ctx.sc.nbdry, n[2], n[0])

    def _checked(self, p, U, B, host: bool):
        """The library copies whole FABs of patch_shapes(p): refuse arrays of
        another shape, type or layout before any copy."""
        ushape, bshape = self.patch_shapes(p)
        for x, shape, what in ((U, ushape, "U"), (B, bshape, "B")):
            if x is None:
                continue
            if tuple(x.shape) != shape:
                raise ValueError(f"patch {p}: {what} has shape {tuple(x.shape)}, expected {shape}")
            if host:
                if not isinstance(x, np.ndarray) or x.dtype != np.float64 or not x.flags.c_contiguous:
                    raise ValueError(f"patch {p}: {what} must be a C-contiguous float64 numpy array")
            elif x.dtype != _torch().float64 or not x.is_cuda or not x.is_contiguous():
                raise ValueError(f"patch {p}: {what} must be a contiguous float64 CUDA tensor")

    def set_patch(self, p, U, B=None):
        """U (and B on the fault plane): numpy arrays (host) or CUDA tensors
        (device) of patch_shapes(p)."""
        host = isinstance(U, np.ndarray)
        if host:
            U = np.ascontiguousarray(U, dtype=np.float64)
            B = np.ascontiguousarray(B, dtype=np.float64) if B is not None else None
        self._checked(p, U, B, host)
        ptr = (lambda x: x.ctypes.data) if host else (lambda x: x.data_ptr())
        A.check(self.lib.tmk_level3d_set_patch(self.h, p, ptr(U), ptr(B) if B is not None else None, int(host)),
                "tmk_level3d_set_patch")

    def get_patch(self, p, U=None, B=None):
        """Copy out one patch (into numpy arrays allocated here if not given)."""
        ushape, bshape = self.patch_shapes(p)
        if U is None:
            U = np.empty(ushape)
        if B is None and self.touches_fault(p):
            B = np.empty(bshape)
        host = isinstance(U, np.ndarray)
        self._checked(p, U, B, host)
        ptr = (lambda x: x.ctypes.data) if host else (lambda x: x.data_ptr())
        A.check(self.lib.tmk_level3d_get_patch(self.h, p, ptr(U), ptr(B) if B is not None else None, int(host)),
                "tmk_level3d_get_patch")
        return U, B

    def exchange(self, stream=None):
        A.check(self.lib.tmk_level3d_exchange(self.h, _stream_ptr(stream)), "tmk_level3d_exchange")

    def step(self, t: float, dt: float, stream=None) -> float:
        mws = C.c_double(0.0)
        A.check(self.lib.tmk_level3d_step(self.h, t, dt, C.byref(mws), _stream_ptr(stream)), "tmk_level3d_step")
        return mws.value

    def close(self):
        if self.h:
            self.lib.tmk_level3d_destroy(self.h)
            self.h = None


class LinElastLevelGodunov:
    """Device-resident single level (all patches of the level in one launch)."""

    def __init__(self, ctx: Context, boxes, domain=None, dx: float | None = None):
        self.ctx = ctx
        sc = ctx.sc
        self.boxes = [tuple(b) for b in boxes]
        self.domain = domain or (0, 0, sc.nx - 1, sc.ny - 1)
        self.dx = sc.dx if dx is None else dx
        self.lib = ctx.lib
        arr = (A.Box * len(self.boxes))(*[A.box(*b) for b in self.boxes])
        h = C.c_void_p()
        A.check(self.lib.tmk_level_create(ctx.h, C.byref(A.box(*self.domain)), self.dx, len(self.boxes), arr,
                                          C.byref(h)), "tmk_level_create")
        self.h = h
        self.pdomains = [self.domain] * len(self.boxes)

    def patch_shapes(self, p):
        b = self.boxes[p]
        g = A.TMK_NGHOST
        ushape = (22, b[3] - b[1] + 1 + 2 * g, b[2] - b[0] + 1 + 2 * g)
        bshape = (self.ctx.sc.nbdry, b[2] - b[0] + 1 + 2 * g)
        return ushape, bshape

    def touches_fault(self, p) -> bool:
        return self.ctx.sc.scheme.fault_law != A.TMK_FAULT_NONE and self.boxes[p][1] == self.pdomains[p][1]

    def set_patch(self, p, U, B=None):
        """U: (22, ny+8, nx+8) float64 over the patch grown by 4 ghosts; numpy
        (host) or CUDA tensor (device)."""
        host = isinstance(U, np.ndarray)
        if host:
            U = np.ascontiguousarray(U, dtype=np.float64)
            Bp = np.ascontiguousarray(B, dtype=np.float64) if B is not None else None
            A.check(self.lib.tmk_level_set_patch(self.h, p, U.ctypes.data, Bp.ctypes.data if Bp is not None else None,
                                                 1), "tmk_level_set_patch")
        else:
            A.check(self.lib.tmk_level_set_patch(self.h, p, U.data_ptr(), B.data_ptr() if B is not None else None,
                                                 0), "tmk_level_set_patch")

    def get_patch(self, p, U=None, B=None):
        """Copy out one patch (into numpy arrays allocated here if not given)."""
        ushape, bshape = self.patch_shapes(p)
        if U is None:
            U = np.empty(ushape)
        if B is None and self.touches_fault(p):
            B = np.empty(bshape)
        host = isinstance(U, np.ndarray)
        uptr = U.ctypes.data if host else U.data_ptr()
        bptr = None
        if B is not None:
            bptr = B.ctypes.data if isinstance(B, np.ndarray) else B.data_ptr()
        A.check(self.lib.tmk_level_get_patch(self.h, p, uptr, bptr, 1 if host else 0), "tmk_level_get_patch")
        return U, B

    def set_fault_friction(self, p, F):
        """Per-face rate-and-state a, b, L of fault patch p: F (3, nx+8) over the
        patch's fault row grown by 4 ghosts (numpy or CUDA tensor)."""
        if isinstance(F, np.ndarray):
            F = np.ascontiguousarray(F, dtype=np.float64)
            A.check(self.lib.tmk_level_set_fault_friction(self.h, p, F.ctypes.data, 1), "tmk_level_set_fault_friction")
        else:
            A.check(self.lib.tmk_level_set_fault_friction(self.h, p, F.data_ptr(), 0), "tmk_level_set_fault_friction")

    def get_fault_friction(self, p):
        """Per-face a, b, L of fault patch p (3, nx+8), or None if not set."""
        if not self.touches_fault(p):
            return None
        _, bshape = self.patch_shapes(p)
        F = np.empty((3, bshape[1]))
        present = C.c_int(0)
        A.check(self.lib.tmk_level_get_fault_friction(self.h, p, F.ctypes.data, 1, C.byref(present)),
                "tmk_level_get_fault_friction")
        return F if present.value else None

    def _ptr(self, a):
        return (a.ctypes.data if isinstance(a, np.ndarray) else a.data_ptr()) if a is not None else None

    def put_valid(self, p, U, B=None):
        """Copy in what a step reads of patch p: the evolving components (and on a
        plastic level lambda, gamma) of the valid cells of U (laid out as for
        set_patch), and B; the level must have had a whole state set once."""
        host = isinstance(U, np.ndarray)
        A.check(self.lib.tmk_level_put_valid(self.h, p, self._ptr(U), self._ptr(B), 1 if host else 0),
                "tmk_level_put_valid")

    def take_valid(self, p, U, B=None):
        """Copy out what a step rewrites of patch p into U (and B); the other
        components and the ghost cells of U are left as they are."""
        host = isinstance(U, np.ndarray)
        A.check(self.lib.tmk_level_take_valid(self.h, p, self._ptr(U), self._ptr(B), 1 if host else 0),
                "tmk_level_take_valid")

    def set_level_friction(self, Fg: np.ndarray):
        """Scatter a domain-wide per-face friction row (3, nx+8) into the fault patches."""
        g = A.TMK_NGHOST
        for p, b in enumerate(self.boxes):
            if self.touches_fault(p):
                dom = self.pdomains[p]
                self.set_fault_friction(p, Fg[:, b[0] - dom[0]:b[2] - dom[0] + 1 + 2 * g])

    def _scatter(self, patches, dom, Ug, Bg):
        g = A.TMK_NGHOST
        for p in patches:
            b = self.boxes[p]
            U = np.ascontiguousarray(Ug[:, b[1] - dom[1]:b[3] - dom[1] + 1 + 2 * g,
                                        b[0] - dom[0]:b[2] - dom[0] + 1 + 2 * g])
            B = None
            if self.touches_fault(p):
                B = np.ascontiguousarray(Bg[:, b[0] - dom[0]:b[2] - dom[0] + 1 + 2 * g])
            self.set_patch(p, U, B)

    def _gather(self, patches, dom, Ug, Bg):
        g = A.TMK_NGHOST
        for p in patches:
            b = self.boxes[p]
            U, B = self.get_patch(p)
            ys = slice(b[1] - dom[1] + g, b[3] - dom[1] + 1 + g)
            xs = slice(b[0] - dom[0] + g, b[2] - dom[0] + 1 + g)
            Ug[:, ys, xs] = U[:, g:-g, g:-g]
            if B is not None and Bg is not None:
                Bg[:, xs] = B[:, g:-g]

    def set_level(self, Ug: np.ndarray, Bg: np.ndarray | None):
        """Scatter a domain-wide state (22, ny+8, nx+8) / fault row (nb, nx+8) into the patches."""
        self._scatter(range(len(self.boxes)), self.domain, Ug, Bg)

    def get_level(self, Ug: np.ndarray, Bg: np.ndarray | None):
        """Gather the valid cells of every patch into domain-wide arrays (in place)."""
        self._gather(range(len(self.boxes)), self.domain, Ug, Bg)

    def step(self, time: float, dt: float, stream=None, t_coarse_old: float | None = None,
             t_coarse_new: float | None = None) -> float:
        """LinElastLevelGodunov::step; a level with a coarser level also needs the
        coarse level's old and new times (the coarse-fine time interpolation)."""
        dtn = C.c_double(0.0)
        if t_coarse_old is None:
            A.check(self.lib.tmk_level_step(self.h, time, dt, _stream_ptr(stream), C.byref(dtn)), "tmk_level_step")
        else:
            A.check(self.lib.tmk_level_step_cf(self.h, time, dt, t_coarse_old, t_coarse_new, _stream_ptr(stream),
                                               C.byref(dtn)), "tmk_level_step_cf")
        return dtn.value

    # -------------------------------------------------- coarse-fine coupling
    def attach_coarser(self, coarse: "LinElastLevelGodunov", ref_ratio: int):
        A.check(self.lib.tmk_level_attach_coarser(self.h, coarse.h, ref_ratio), "tmk_level_attach_coarser")

    def detach_coarser(self):
        A.check(self.lib.tmk_level_detach_coarser(self.h), "tmk_level_detach_coarser")

    def fill_coarse_fine(self, alpha: float, stream=None):
        """PiecewiseLinearFillPatch / D1PiecewiseLinearFillPatch::fillInterp."""
        A.check(self.lib.tmk_level_fill_coarse_fine(self.h, alpha, _stream_ptr(stream)), "tmk_level_fill_coarse_fine")

    def reflux(self, stream=None):
        """LevelFluxRegister::reflux with the finer level's fluxes."""
        A.check(self.lib.tmk_level_reflux(self.h, _stream_ptr(stream)), "tmk_level_reflux")

    def average_down(self, stream=None):
        """CoarseAverage / D1CoarseAverage::averageToCoarse from the finer level."""
        A.check(self.lib.tmk_level_average_down(self.h, _stream_ptr(stream)), "tmk_level_average_down")

    def interp_from_coarser(self, stream=None):
        """FineInterp / D1FineInterp::interpToFine (regrid initialisation)."""
        A.check(self.lib.tmk_level_interp_from_coarser(self.h, _stream_ptr(stream)), "tmk_level_interp_from_coarser")

    def copy_overlap(self, src: "LinElastLevelGodunov", stream=None):
        """Copy the valid cells that this level's patches share with `src`'s."""
        A.check(self.lib.tmk_level_copy_overlap(self.h, src.h, _stream_ptr(stream)), "tmk_level_copy_overlap")

    def tag_cells(self, tp, mask=None, stream=None):
        """AMRLevelLinElast::tagCells / tagCellsInit on the device: the tag mask
        over the level's domain, (ny, nx) uint8 (numpy, or a CUDA uint8 tensor
        given as `mask`)."""
        d = self.domain
        if mask is None:
            mask = np.zeros((d[3] - d[1] + 1, d[2] - d[0] + 1), dtype=np.uint8)
        host = isinstance(mask, np.ndarray)
        ptr = mask.ctypes.data if host else mask.data_ptr()
        A.check(self.lib.tmk_level_tag_cells(self.h, C.byref(tp), ptr, 1 if host else 0, _stream_ptr(stream)),
                "tmk_level_tag_cells")
        return mask

    def register_size(self) -> int:
        n = C.c_int(0)
        A.check(self.lib.tmk_level_register_size(self.h, C.byref(n)), "tmk_level_register_size")
        return n.value

    def set_patches(self, Us, Bs):
        """Per-patch state: Us[p] (22, ny+8, nx+8), Bs[p] fault row or None."""
        for p, U in enumerate(Us):
            self.set_patch(p, U, Bs[p])

    def get_patches(self):
        Us, Bs = [], []
        for p in range(len(self.boxes)):
            U, B = self.get_patch(p)
            Us.append(U)
            Bs.append(B)
        return Us, Bs

    def status(self):
        info = (C.c_longlong * 3)()
        rc = self.lib.tmk_level_status(self.h, info)
        return rc, list(info)

    def launches_per_step(self) -> int:
        return self.lib.tmk_level_launches_per_step(self.h)

    def graph(self, nsteps: int, time: float, dt: float) -> "StepGraph":
        """Record `nsteps` (even) steps as one CUDA graph (nothing runs yet)."""
        h = C.c_void_p()
        A.check(self.lib.tmk_level_graph_create(self.h, nsteps, time, dt, C.byref(h)), "tmk_level_graph_create")
        return StepGraph(self.lib, h)

    def tuning(self) -> A.Tuning:
        t = A.Tuning()
        A.check(self.lib.tmk_level_get_tuning(self.h, C.byref(t)), "tmk_level_get_tuning")
        return t

    def set_tuning(self, t: A.Tuning):
        """Work-list shape and kernel variants (rebuilds the work lists)."""
        A.check(self.lib.tmk_level_set_tuning(self.h, C.byref(t)), "tmk_level_set_tuning")

    def autotune(self, time: float, dt: float, steps: int = 8, stream=None):
        """Time the candidate tunings on the level's present state, keep the
        fastest and put the state back.  Returns (tuning, ms per step)."""
        t = A.Tuning()
        ms = C.c_double(0.0)
        A.check(self.lib.tmk_level_autotune(self.h, time, dt, steps, _stream_ptr(stream), C.byref(t), C.byref(ms)),
                "tmk_level_autotune")
        return t, ms.value

    def profile(self, enable: bool, max_steps: int = 0):
        A.check(self.lib.tmk_level_profile(self.h, int(enable), max_steps), "tmk_level_profile")

    def profile_read(self):
        """Average ms per step: (exchange, fault kernel, volume kernel, whole step), nsteps."""
        out = (C.c_double * 4)()
        n = C.c_int(0)
        A.check(self.lib.tmk_level_profile_read(self.h, out, C.byref(n)), "tmk_level_profile_read")
        return list(out), n.value

    def close(self):
        if self.h:
            self.lib.tmk_level_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class LinElastEnsemble(LinElastLevelGodunov):
    """Independent scenarios stepped together as one level (tmk_ensemble_create):
    scenario k has its own context (friction parameters), problem domain and
    patches; every kernel of a step covers all of them.  The reference runs one
    scenario per process; this is an extension."""

    def __init__(self, ctxs, domains, boxes, dx: float | None = None):
        """ctxs[k], domains[k] = (xlo, ylo, xhi, yhi) and boxes[k] (a list of
        patch boxes) per scenario k."""
        self.ctxs = list(ctxs)
        self.ctx = self.ctxs[0]
        self.lib = self.ctx.lib
        self.dx = self.ctx.sc.dx if dx is None else dx
        self.domains = [tuple(d) for d in domains]
        self.domain = self.domains[0]
        self.boxes, self.scen = [], []
        for k, bk in enumerate(boxes):
            for b in bk:
                self.boxes.append(tuple(b))
                self.scen.append(k)
        self.pdomains = [self.domains[k] for k in self.scen]
        n = len(self.boxes)
        harr = (C.c_void_p * len(self.ctxs))(*[c.h for c in self.ctxs])
        darr = (A.Box * len(self.domains))(*[A.box(*d) for d in self.domains])
        barr = (A.Box * n)(*[A.box(*b) for b in self.boxes])
        sarr = (C.c_int * n)(*self.scen)
        h = C.c_void_p()
        self.h = None
        A.check(self.lib.tmk_ensemble_create(len(self.ctxs), harr, darr, self.dx, n, barr, sarr, C.byref(h)),
                "tmk_ensemble_create")
        self.h = h

    def patches_of(self, k):
        return [p for p, s in enumerate(self.scen) if s == k]

    def set_scenario(self, k, Ug: np.ndarray, Bg: np.ndarray | None):
        """Scatter scenario k's domain-wide state into its patches."""
        self._scatter(self.patches_of(k), self.domains[k], Ug, Bg)

    def get_scenario(self, k, Ug: np.ndarray, Bg: np.ndarray | None):
        """Gather scenario k's valid cells into domain-wide arrays (in place)."""
        self._gather(self.patches_of(k), self.domains[k], Ug, Bg)

    def cells(self) -> int:
        return sum((b[2] - b[0] + 1) * (b[3] - b[1] + 1) for b in self.boxes)


class StepGraph:
    """Recorded steps of a level or an AMR hierarchy (tmk_graph)."""

    def __init__(self, lib, h):
        self.lib = lib
        self.h = h

    def launch(self, time: float, stream=None):
        """Replay the recorded steps starting at `time`."""
        A.check(self.lib.tmk_graph_launch(self.h, time, _stream_ptr(stream)), "tmk_graph_launch")

    def close(self):
        if self.h:
            self.lib.tmk_graph_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
