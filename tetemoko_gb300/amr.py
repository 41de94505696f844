"""Subcycled AMR hierarchy over device levels (Chombo AMR::timeStep driving
AMRLevelLinElast::advance / postTimeStep, srcLinElast/AMRLevelLinElast.cpp:420-515).

Each level is a LinElastLevelGodunov (device-resident patches).  Creating the
hierarchy attaches level l+1 to level l with ratios[l]; one `step(dt0)`
advances level 0 by dt0, every finer level by its ratio's share in substeps
(coarse-fine ghost fill with time interpolation, flux registers), and then
refluxes and averages down.  `regrid_level` gives the device half of a regrid
(prolongation from the coarser level, then the copy of the old level's
overlapping cells); `boxes_from_tags` and `regrid` give a caller without
Chombo the host half (tags from the device, boxes by Berger-Rigoutsos
clustering).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _capi as A
from .level import LinElastLevelGodunov, StepGraph, _stream_ptr


def refine_domain(domain, r: int):
    """Domain of the next finer level (cell indices, inclusive)."""
    return (domain[0] * r, domain[1] * r, (domain[2] + 1) * r - 1, (domain[3] + 1) * r - 1)


def refine_box(box, r: int):
    return (box[0] * r, box[1] * r, (box[2] + 1) * r - 1, (box[3] + 1) * r - 1)


class AMRHierarchy:
    def __init__(self, levels: list[LinElastLevelGodunov], ratios: list[int], time: float = 0.0):
        self.levels = list(levels)
        self.ratios = list(ratios)
        self.lib = A.lib()
        n = len(self.levels)
        arr = (C.c_void_p * n)(*[lv.h.value for lv in self.levels])
        rat = (C.c_int * max(1, n - 1))(*(self.ratios or [1]))
        h = C.c_void_p()
        A.check(self.lib.tmk_amr_create(n, arr, rat, time, C.byref(h)), "tmk_amr_create")
        self.h = h

    def step(self, dt0: float, stream=None):
        A.check(self.lib.tmk_amr_step(self.h, dt0, _stream_ptr(stream)), "tmk_amr_step")

    def autotune(self, dt0: float, ncoarse: int = 2, stream=None):
        """Pick every level's tuning by timing whole subcycled coarse steps
        (levels one at a time, finest first); the hierarchy's state and clock
        are put back.  Returns (tunings per level, ms per coarse step)."""
        n = len(self.levels)
        out = (A.Tuning * n)()
        ms = C.c_double(0.0)
        A.check(self.lib.tmk_amr_autotune(self.h, dt0, ncoarse, _stream_ptr(stream), out, C.byref(ms)),
                "tmk_amr_autotune")
        return [out[k] for k in range(n)], ms.value

    def time(self, level: int = 0) -> float:
        t = C.c_double(0.0)
        A.check(self.lib.tmk_amr_time(self.h, level, C.byref(t)), "tmk_amr_time")
        return t.value

    def cell_updates(self) -> int:
        """Cell-updates of one step: sum over levels of valid cells x substeps."""
        return int(self.lib.tmk_amr_cell_updates(self.h))

    def launches_per_step(self) -> int:
        return int(self.lib.tmk_amr_launches_per_step(self.h))

    def graph(self, ncoarse: int, dt0: float) -> StepGraph:
        """Record `ncoarse` (even) subcycled coarse steps as one CUDA graph from
        the current time; StepGraph.launch(t) replays them from time t."""
        h = C.c_void_p()
        A.check(self.lib.tmk_amr_graph_create(self.h, ncoarse, dt0, C.byref(h)), "tmk_amr_graph_create")
        return StepGraph(self.lib, h)

    def close(self):
        if self.h:
            self.lib.tmk_amr_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def regrid_level(new: LinElastLevelGodunov, old: LinElastLevelGodunov | None, coarse: LinElastLevelGodunov,
                 ratio: int, stream=None):
    """AMRLevelLinElast::regrid (srcLinElast/AMRLevelLinElast.cpp:900-946) on the
    device: attach `new` to `coarse`, fill its valid cells from the coarse level
    (FineInterp / D1FineInterp), then copy the cells `old` shares with it."""
    new.attach_coarser(coarse, ratio)
    new.interp_from_coarser(stream)
    if old is not None:
        new.copy_overlap(old, stream)


# ------------------------------------------------------------------ regrid
def _cluster(tags: np.ndarray, fill_ratio: float, allowed: np.ndarray | None):
    """Berger & Rigoutsos (1991) clustering of a boolean mask (y, x): boxes
    (x0, y0, x1, y1) covering every tag, each at least `fill_ratio` tagged
    (or a single cell), split at a hole of the tag signature nearest the box
    centre, else at the strongest inflection of its Laplacian, else in half
    along the longer side.  With `allowed`, a box holding a cell outside it is
    split further; a single such cell is dropped."""
    out = []
    ys, xs = np.nonzero(tags)
    if len(xs) == 0:
        return out
    stack = [(xs.min(), ys.min(), xs.max(), ys.max())]
    while stack:
        x0, y0, x1, y1 = stack.pop()
        sub = tags[y0:y1 + 1, x0:x1 + 1]
        if not sub.any():
            continue
        ys, xs = np.nonzero(sub)                      # shrink to the tags' bounding box
        x0, x1, y0, y1 = x0 + xs.min(), x0 + xs.max(), y0 + ys.min(), y0 + ys.max()
        sub = tags[y0:y1 + 1, x0:x1 + 1]
        bad = allowed is not None and not allowed[y0:y1 + 1, x0:x1 + 1].all()
        if not bad and sub.sum() >= fill_ratio * sub.size:
            out.append((x0, y0, x1, y1))
            continue
        nx, ny = x1 - x0 + 1, y1 - y0 + 1
        if nx == 1 and ny == 1:
            if not bad:
                out.append((x0, y0, x1, y1))
            continue
        cut = None                                    # (direction, first index of the upper part)
        best = None
        for d, sig in ((0, sub.sum(axis=0)), (1, sub.sum(axis=1))):
            n = len(sig)
            holes = [i for i in range(1, n - 1) if sig[i] == 0]
            if holes:
                i = min(holes, key=lambda k: abs(k - (n - 1) / 2))
                score = (2, -abs(i - (n - 1) / 2))
                if best is None or score > best:
                    best, cut = score, (d, i)
        if cut is None:
            for d, sig in ((0, sub.sum(axis=0)), (1, sub.sum(axis=1))):
                n = len(sig)
                if n < 4:
                    continue
                lap = sig[2:] - 2 * sig[1:-1] + sig[:-2]          # at indices 1..n-2
                for k in range(1, len(lap)):
                    if lap[k - 1] * lap[k] < 0:
                        jump = abs(int(lap[k]) - int(lap[k - 1]))
                        score = (1, jump)
                        if best is None or score > best:
                            best, cut = score, (d, k + 1)
        if cut is None:
            cut = (0, nx // 2) if nx >= ny else (1, ny // 2)
        d, i = cut
        if d == 0:
            stack.append((x0, y0, x0 + i - 1, y1))
            stack.append((x0 + i, y0, x1, y1))
        else:
            stack.append((x0, y0, x1, y0 + i - 1))
            stack.append((x0, y0 + i, x1, y1))
    return out


def _split(box, maxn):
    """Split a box into nearly equal pieces no longer than maxn cells per side."""
    x0, y0, x1, y1 = box
    nxp = -(-(x1 - x0 + 1) // maxn)
    nyp = -(-(y1 - y0 + 1) // maxn)
    xe = np.linspace(x0, x1 + 1, nxp + 1).round().astype(int)
    ye = np.linspace(y0, y1 + 1, nyp + 1).round().astype(int)
    return [(int(xe[a]), int(ye[b]), int(xe[a + 1]) - 1, int(ye[b + 1]) - 1) for b in range(nyp) for a in range(nxp)]


def boxes_from_tags(mask: np.ndarray, domain, ratio: int, block_factor: int = 8, max_grid_size: int = 128,
                    fill_ratio: float = 0.75, nest_boxes=None, nest_buffer: int = 1):
    """Boxes of the next finer level from the tags of this level (the host
    half of a regrid, which Chombo's BRMeshRefine does for the reference).

    mask (ny, nx) over `domain` (xlo, ylo, xhi, yhi); the new boxes are in the
    finer level's cells, multiples of `block_factor` fine cells, at most
    `max_grid_size` per side, and properly nested: inside `nest_boxes` (this
    level's patches; None = the whole domain) shrunk by `nest_buffer` cells
    away from the domain's edges.  Tags are coarsened by block_factor/ratio
    (at least 1) cells, clustered (Berger & Rigoutsos), refined back."""
    ny, nx = mask.shape
    bf = max(1, block_factor // ratio)
    if nx % bf or ny % bf or domain[0] % bf or domain[1] % bf:
        raise ValueError("domain not aligned to the coarsened blocking factor")
    allowed = np.zeros((ny, nx), dtype=bool)
    if nest_boxes is None:
        allowed[:] = True
    else:
        for b in nest_boxes:
            x0, y0, x1, y1 = (b[0] - domain[0], b[1] - domain[1], b[2] - domain[0], b[3] - domain[1])
            allowed[y0:y1 + 1, x0:x1 + 1] = True
        if nest_buffer > 0:       # shrink the union, except against the domain's edges
            pad = np.pad(allowed, nest_buffer, mode="edge")
            shr = np.ones_like(allowed)
            for dy in range(-nest_buffer, nest_buffer + 1):
                for dx in range(-nest_buffer, nest_buffer + 1):
                    shr &= pad[nest_buffer + dy:nest_buffer + dy + ny, nest_buffer + dx:nest_buffer + dx + nx]
            allowed = shr
    tags = mask.astype(bool) & allowed
    # blocks of bf x bf cells: tagged if any cell is, allowed if every cell is
    tb = tags.reshape(ny // bf, bf, nx // bf, bf).any(axis=(1, 3))
    ab = allowed.reshape(ny // bf, bf, nx // bf, bf).all(axis=(1, 3))
    maxb = max(1, max_grid_size // (ratio * bf))
    out = []
    for (x0, y0, x1, y1) in _cluster(tb, fill_ratio, ab):
        for (a0, b0, a1, b1) in _split((x0, y0, x1, y1), maxb):
            box = ((a0 * bf + domain[0]) * ratio, (b0 * bf + domain[1]) * ratio,
                   ((a1 + 1) * bf + domain[0]) * ratio - 1, ((b1 + 1) * bf + domain[1]) * ratio - 1)
            out.append(box)
    return out


def regrid(levels: list[LinElastLevelGodunov], ratios: list[int], tag_params, max_level: int | None = None,
           stream=None, **box_args):
    """One regrid of a hierarchy, coarse to fine (AMR::regrid over
    AMRLevelLinElast::tagCells / regrid): tags of level l on the device, boxes
    of level l+1 from them (boxes_from_tags, nested in the new level l), a new
    level l+1 prolonged from the new level l and given the old level's cells
    where they overlap.  tag_params: one A.TagParams per level that may be
    refined.  Returns the new level list (level 0 kept; the old finer levels
    are left to the caller to close).  Close the old AMRHierarchy and its
    graphs first; the caller builds a new AMRHierarchy from the result and
    gives the new levels their per-level settings (per-face friction,
    stations, tuning)."""
    nlev = len(levels) if max_level is None else max_level + 1
    new = [levels[0]]
    for l in range(nlev - 1):
        base = new[l]
        mask = base.tag_cells(tag_params[l], stream=stream)
        r = ratios[l]
        boxes = boxes_from_tags(mask, base.domain, r, nest_boxes=base.boxes if l > 0 else None, **box_args)
        if not boxes:
            break
        lv = LinElastLevelGodunov(base.ctx, boxes, domain=refine_domain(base.domain, r), dx=base.dx / r)
        old = levels[l + 1] if l + 1 < len(levels) else None
        regrid_level(lv, old, base, r, stream)      # attaching replaces base's previous finer level
        new.append(lv)
    return new
