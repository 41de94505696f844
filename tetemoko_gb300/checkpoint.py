"""Checkpoint and restart of device levels (the reference's
writeCheckpointLevel / readCheckpointLevel, srcLinElast/AMRLevelLinElast.cpp:
1126-1400, stage U and B through the host into Chombo's HDF5 files; h5py is
not part of this image, so the same content goes to one numpy .npz archive).

A checkpoint holds the scenario's parameter structs, and per level its domain,
dx, patch boxes, every patch's state and fault data, per-face friction and
tuning, plus the hierarchy's ratios and time.  Taken between coarse steps (all
levels at the same time), a restart continues bit for bit: the ghost cells a
step reads are refilled by exchange and the coarse-fine fill, and the other
state buffer is rewritten by the first step.  A 3-D device level
(save_3d / load_3d) keeps its scenario, boxes and every patch's whole FABs.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _capi as A
from .scenarios import Scenario


def _struct_bytes(s):
    return np.frombuffer(bytes(s), dtype=np.uint8) if s is not None else np.zeros(0, dtype=np.uint8)


def _struct_from(cls, arr):
    return cls.from_buffer_copy(arr.tobytes()) if arr.size else None


def _scenario_arrays(sc: Scenario) -> dict:
    return {"name": np.array(sc.name), "grid": np.array([sc.nx, sc.ny]), "dx_cfl": np.array([sc.dx, sc.cfl]),
            "elastic": _struct_bytes(sc.elastic), "scheme": _struct_bytes(sc.scheme), "rs": _struct_bytes(sc.rs),
            "sw": _struct_bytes(sc.sw), "plastic": _struct_bytes(sc.plastic)}


def _scenario_from(z) -> Scenario:
    nx, ny = (int(v) for v in z["grid"])
    dx, cfl = (float(v) for v in z["dx_cfl"])
    return Scenario(str(z["name"]), nx, ny, dx, cfl, _struct_from(A.ElasticParams, z["elastic"]),
                    _struct_from(A.Scheme, z["scheme"]), _struct_from(A.RSParams, z["rs"]),
                    _struct_from(A.SWParams, z["sw"]), _struct_from(A.PlasticParams, z["plastic"]))


def save(path: str, sc: Scenario, levels, ratios=(), time: float = 0.0):
    """Write `levels` (LinElastLevelGodunov, coarse to fine) and the scenario."""
    out = _scenario_arrays(sc)
    out.update({"ratios": np.array(list(ratios), dtype=np.int64), "time": np.array(time),
                "nlev": np.array(len(levels))})
    for l, lv in enumerate(levels):
        out[f"L{l}_domain"] = np.array(lv.domain)
        out[f"L{l}_dx"] = np.array(lv.dx)
        out[f"L{l}_boxes"] = np.array(lv.boxes, dtype=np.int64)
        out[f"L{l}_tuning"] = _struct_bytes(lv.tuning())
        Us, Bs = lv.get_patches()
        for p in range(len(lv.boxes)):
            out[f"L{l}_U{p}"] = Us[p]
            if Bs[p] is not None:
                out[f"L{l}_B{p}"] = Bs[p]
                F = lv.get_fault_friction(p)
                if F is not None:
                    out[f"L{l}_F{p}"] = F
    np.savez(path, **out)


def load(path: str):
    """Rebuild the scenario, a context and the levels of a checkpoint (levels
    attached coarse to fine).  Returns (scenario, context, levels, ratios, time);
    build an AMRHierarchy(levels, ratios, time) to continue a hierarchy."""
    with np.load(path) as z:
        return _rebuild(z)


def _rebuild(z):
    from .level import Context, LinElastLevelGodunov
    sc = _scenario_from(z)
    ctx = Context(sc)
    ratios = [int(r) for r in z["ratios"]]
    levels = []
    for l in range(int(z["nlev"])):
        boxes = [tuple(int(v) for v in b) for b in z[f"L{l}_boxes"]]
        lv = LinElastLevelGodunov(ctx, boxes, domain=tuple(int(v) for v in z[f"L{l}_domain"]),
                                  dx=float(z[f"L{l}_dx"]))
        for p in range(len(boxes)):
            lv.set_patch(p, z[f"L{l}_U{p}"], z[f"L{l}_B{p}"] if f"L{l}_B{p}" in z else None)
            if f"L{l}_F{p}" in z:
                lv.set_fault_friction(p, z[f"L{l}_F{p}"])
        lv.set_tuning(_struct_from(A.Tuning, z[f"L{l}_tuning"]))
        if l > 0:
            lv.attach_coarser(levels[l - 1], ratios[l - 1])
        levels.append(lv)
    return sc, ctx, levels, ratios, float(z["time"])


def save_3d(path: str, sc: Scenario, level, time: float = 0.0):
    """Write a 3-D device level (LinElastLevelGodunov3D) and the scenario: its
    domain, dx, patch boxes and every patch's whole state and fault-data FABs."""
    out = _scenario_arrays(sc)
    out.update({"dim": np.array(3), "time": np.array(time), "domain3": np.array(level.domain, dtype=np.int64),
                "dx3": np.array(level.dx), "boxes3": np.array(level.boxes, dtype=np.int64)})
    for p in range(len(level.boxes)):
        U, B = level.get_patch(p)
        out[f"U{p}"] = U
        if B is not None:
            out[f"B{p}"] = B
    np.savez(path, **out)


def load_3d(path: str):
    """Rebuild the scenario, a context and the 3-D level of a save_3d archive.
    Returns (scenario, context, level, time)."""
    from .level import Context, LinElastLevelGodunov3D
    with np.load(path) as z:
        sc = _scenario_from(z)
        ctx = Context(sc)
        boxes = [tuple(tuple(int(v) for v in corner) for corner in b) for b in z["boxes3"]]
        domain = tuple(tuple(int(v) for v in corner) for corner in z["domain3"])
        level = LinElastLevelGodunov3D(ctx, boxes, domain, dx=float(z["dx3"]))
        for p in range(len(boxes)):
            level.set_patch(p, z[f"U{p}"], z[f"B{p}"] if f"B{p}" in z else None)
        return sc, ctx, level, float(z["time"])
