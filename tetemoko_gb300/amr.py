"""Subcycled AMR hierarchy over device levels (Chombo AMR::timeStep driving
AMRLevelLinElast::advance / postTimeStep, srcLinElast/AMRLevelLinElast.cpp:420-515).

Each level is a LinElastLevelGodunov (device-resident patches).  Creating the
hierarchy attaches level l+1 to level l with ratios[l]; one `step(dt0)`
advances level 0 by dt0, every finer level by its ratio's share in substeps
(coarse-fine ghost fill with time interpolation, flux registers), and then
refluxes and averages down.  Box generation (tagging, regrid) stays with the
caller; `regrid_level` gives the device half of a regrid (prolongation from
the coarser level, then the copy of the old level's overlapping cells).
"""
from __future__ import annotations

import ctypes as C

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
