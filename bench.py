#!/usr/bin/env python
"""Benchmark of the per-level Godunov step on the rate-and-state fault workload.

Workload: planar rate-and-state fault on a uniform 2048 x 1024 grid, dx = 0.1 km
(aging law, regularised sinh friction, Gaussian 25 MPa nucleation), one level,
synthetic initial data as the reference's initialisers set it.  A step is one
LinElastLevelGodunov::step of the whole level.

Reported (one JSON line, rank 0):
  value        mixed form (FP32 volume, FP64 fault) cell-updates/s, state resident in HBM
  fp64_plain   the plain FP64 form on the same workload
  roofline     volume kernel: algorithmic bytes (18 components read + written, 144 B per
               cell in FP32) / average launch time from CUDA events on the launch stream
  e2e          the same step through the C ABI with the state in a host (pinned) FP64 FAB:
               every step copies in what the step reads and copies out what it rewrites
  cpu_baseline the CPU oracle (a port of the reference) on the machine's host cores
With --gpus N > 1 (torchrun) every rank runs an independent replica ("replicas
only": the level step has no data-path collective on one GPU per box).
`--impl reference` times the reference's CPU path (the oracle port) instead.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

NX, NY = 2048, 1024
METRIC = "cell-updates/s (rate-and-state level step, mixed FP32 volume / FP64 fault)"
UNIT = "cell-updates/s"
BYTES_PER_CELL_MIXED = 144   # 18 evolving components read + written, FP32
BYTES_PER_CELL_FP64 = 288


def workload_config(nx=NX, ny=NY):
    return {
        "workload": f"rate-and-state planar fault, uniform {nx}x{ny}, dx=0.1 km, aging law, "
                    "Gaussian 25 MPa / 3 km nucleation, absorbing edges, PPM + prim limiting, CFL 0.9",
        "cells": nx * ny,
        "precision": "FP32 volume stencil, FP64 friction solve and fault accumulators",
        "l2": "inputs larger than L2 (FP32 state 187 MB per buffer, two buffers)",
        "parallelism": "replicas (one independent level per GPU)",
    }


def rank_env():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def replica_rate(cells: int, steps: int, seconds_local: float, world: int, device=None) -> tuple[float, float]:
    """Whole-job throughput of `world` independent replicas: every rank advanced
    `cells` cells `steps` times; the job took the slowest rank's time.
    Returns (cell-updates/s, max seconds)."""
    t = seconds_local
    if world > 1:
        import torch
        import torch.distributed as dist
        x = torch.tensor([seconds_local], dtype=torch.float64, device=device)
        dist.all_reduce(x, op=dist.ReduceOp.MAX)
        t = float(x.item())
    return world * cells * steps / t, t


class NvmlClockSampler:
    """SM clock and clock-event reasons of this process's GPU, polled through
    NVML (read-only queries) every 20 ms from a thread while the timed loop
    runs; every sample falls inside the timed region."""

    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown",
               0x40: "hw_thermal_slowdown", 0x80: "hw_power_brake_slowdown"}

    def __init__(self, device_index=0):
        import ctypes
        import threading
        self.ct = ctypes
        self.nv = ctypes.CDLL("libnvidia-ml.so.1")
        if self.nv.nvmlInit_v2() != 0:
            raise RuntimeError("nvmlInit failed")
        import torch
        uuid = "GPU-" + str(torch.cuda.get_device_properties(device_index).uuid)
        self.h = ctypes.c_void_p()
        if self.nv.nvmlDeviceGetHandleByUUID(uuid.encode(), ctypes.byref(self.h)) != 0:
            raise RuntimeError("no NVML handle for " + uuid)
        self.reason_fn = getattr(self.nv, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            self.nv.nvmlDeviceGetCurrentClocksThrottleReasons
        self.samples = []
        self.stop_evt = threading.Event()
        self.thread = None
        self.threading = threading

    def _poll(self):
        ct = self.ct
        mhz = ct.c_uint(0)
        rs = ct.c_ulonglong(0)
        while not self.stop_evt.is_set():
            if self.nv.nvmlDeviceGetClockInfo(self.h, 1, ct.byref(mhz)) == 0 and \
                    self.reason_fn(self.h, ct.byref(rs)) == 0:
                self.samples.append((mhz.value, rs.value))
            self.stop_evt.wait(0.02)

    def start(self):
        self.samples = []
        self.stop_evt.clear()
        self.thread = self.threading.Thread(target=self._poll, daemon=True)
        self.thread.start()

    def stop(self):
        self.stop_evt.set()
        self.thread.join(timeout=2)
        ct = self.ct
        smax = ct.c_uint(0)
        self.nv.nvmlDeviceGetMaxClockInfo(self.h, 1, ct.byref(smax))
        reasons = set()
        for _, r in self.samples:
            for bit, name in self.REASONS.items():
                if r & bit:
                    reasons.add(name)
        sm = [m for m, _ in self.samples]
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax.value or None,
                "reasons": sorted(reasons), "samples": len(sm), "samples_under_load": len(sm),
                "source": "NVML, 20 ms polling inside the timed region"}


def make_clock_sampler():
    try:
        return NvmlClockSampler()
    except Exception:
        return ClockSampler()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,utilization.gpu,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        with open(self.path) as f:
            for line in f:
                p = [x.strip() for x in line.split(",")]
                if len(p) >= 10:
                    rows.append(p)
        os.unlink(self.path)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        sm, smax = [], None
        for p in rows:
            try:
                util = float(p[4])
                clk = float(p[1])
                smax = float(p[2])
            except ValueError:
                continue
            if util >= 50:
                sm.append(clk)
            for k, n in enumerate(names):
                if p[6 + k].lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(rows), "samples_under_load": len(sm)}


def cpu_sample(sc, max_seconds, nthreads, strip_rows=None):
    """Time the oracle level step on the host cores; returns (cell-updates/s, sample description)."""
    import numpy as np  # noqa: F401
    import oracle as O
    from tetemoko_gb300 import scenarios as S
    rows = strip_rows or sc.ny
    sub = S.rate_state(nx=sc.nx, ny=rows, dx=sc.dx)
    boxes = O.tile_boxes(sub.nx, sub.ny, 128)
    U = sub.initial_U()
    B = sub.initial_B()
    dt = sub.dt()
    t = 0.0
    O.level_step(sub, U, B, boxes, t, dt, nthreads=nthreads)   # warm-up
    t += dt
    n = 0
    t0 = time.perf_counter()
    while True:
        O.level_step(sub, U, B, boxes, t, dt, nthreads=nthreads)
        t += dt
        n += 1
        el = time.perf_counter() - t0
        if el >= max_seconds or n >= 1000:
            break
    rate = sub.nx * sub.ny * n / el
    desc = (f"{n} level steps of a {sub.nx}x{sub.ny} strip of the workload (128x128 patches, OpenMP over "
            f"patches, {nthreads} threads), {el:.1f} s")
    return rate, desc


def tile_boxes(lo0, lo1, hi0, hi1, max_grid):
    """Cover [lo0, hi0] x [lo1, hi1] with boxes of at most max_grid cells per side."""
    out = []
    for j0 in range(lo1, hi1 + 1, max_grid):
        for i0 in range(lo0, hi0 + 1, max_grid):
            out.append((i0, j0, min(i0 + max_grid - 1, hi0), min(j0 + max_grid - 1, hi1)))
    return out


# 4-level hierarchy, ratio 2, base 1024 x 512 (dx 0.1 km, effective 8192 x 4096 at
# 12.5 m): nested bands along the fault around the nucleation (cell boxes per level)
AMR_BASE = (1024, 512)
AMR_REGIONS = [(512, 0, 1535, 255), (1280, 0, 2815, 383), (3072, 0, 5119, 511)]


def amr_measurement(steps, warmup, stream, autotune=True):
    """Subcycled 4-level rate-and-state hierarchy with plasticity, per-face
    friction (a, b, L within 10 % of nominal), a normal stress rising along
    strike from 20 to 120 MPa and the shear prestress in proportion; steps
    replayed from a CUDA graph of 2 coarse steps.  Returns the JSON object of
    the measurement."""
    import numpy as np
    import torch
    from tetemoko_gb300 import _capi as A, scenarios as S
    from tetemoko_gb300.amr import AMRHierarchy, refine_domain
    from tetemoko_gb300.level import Context, LinElastLevelGodunov
    nx, ny = AMR_BASE
    sc = S.rate_state(nx=nx, ny=ny, precision=A.TMK_PREC_MIXED, plasticity=True)
    ctx = Context(sc)
    g = A.TMK_NGHOST
    levels, boxes_all = [], []
    dom = (0, 0, nx - 1, ny - 1)
    dx = sc.dx
    boxes = tile_boxes(0, 0, nx - 1, ny - 1, 128)
    for l in range(4):
        if l > 0:
            dom = refine_domain(dom, 2)
            dx = dx / 2
            boxes = tile_boxes(*AMR_REGIONS[l - 1], 128)
        levels.append(LinElastLevelGodunov(ctx, boxes, domain=dom, dx=dx))
        boxes_all.append(boxes)
    # level 0: background with syy(x) from -20 to -120 MPa along strike
    x = (np.arange(-g, nx + g) + 0.5) / nx
    for p, b in enumerate(boxes_all[0]):
        U = sc.initial_U(lo=b[:2], hi=b[2:])
        xs = np.clip(x[b[0]:b[2] + 2 * g + 1], 0.0, 1.0)
        for side in (0, 11):          # shear keeps the 70/120 ratio of the uniform workload
            U[side + 4] = -(20.0 + 100.0 * xs)[None, :]
            U[side + 6] = (70.0 / 120.0) * (20.0 + 100.0 * xs)[None, :]
        B = sc.initial_B(xlo=b[0], xhi=b[2]) if b[1] == 0 else None
        levels[0].set_patch(p, U, B)
    for l in range(1, 4):        # finer levels from the coarser ones (regrid prolongation)
        levels[l].attach_coarser(levels[l - 1], 2)
        levels[l].interp_from_coarser(stream)
    # a, b, L per fault face: nominal x (1 + U(-0.1, 0.1)), seed 4001, drawn on the
    # base level's faces; finer faces take their coarse face's values
    for l in range(4):
        levels[l].set_level_friction(S.friction_field(sc, seed=4001, amp=0.1, refine=2 ** l))
    torch.cuda.synchronize()
    h = AMRHierarchy(levels, [2, 2, 2])
    dt0 = sc.dt()
    # every level's tuning from the hierarchy autotuner (whole coarse steps
    # timed from the initial state, which it puts back)
    tunings = []
    if autotune:
        ts, _ = h.autotune(dt0, ncoarse=2, stream=stream)
        tunings = [t.as_dict() for t in ts]
    for _ in range(warmup):
        h.step(dt0, stream)
    graph = h.graph(2, dt0)
    t = h.time(0)
    graph.launch(t, stream)
    t += 2 * dt0
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    nrep = max(1, steps // 2)
    e0.record(stream)
    for _ in range(nrep):
        graph.launch(t, stream)
        t += 2 * dt0
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    per_step = h.cell_updates()
    status = [lv.status()[1] for lv in levels]
    cells = [sum((b[2] - b[0] + 1) * (b[3] - b[1] + 1) for b in bx) for bx in boxes_all]
    out = {"value": per_step * 2 * nrep / (ms * 1e-3), "unit": "cell-updates/s",
           "ms_per_coarse_step": ms / (2 * nrep), "coarse_steps": 2 * nrep,
           "cell_updates_per_coarse_step": per_step, "cells_per_level": cells,
           "patches_per_level": [len(b) for b in boxes_all],
           "launches_per_coarse_step": h.launches_per_step(),
           "config": "4 levels, ratio 2, base 1024x512 at dx=0.1 km (finest 12.5 m, effective 8192x4096), "
                     "rate-and-state aging law with a, b, L per fault face = nominal x (1 + U(-0.1, 0.1)) "
                     "(seed 4001, base-level faces, refined piecewise constant), Drucker-Prager plasticity, "
                     "normal stress 20-120 MPa along strike, FP32 volume / FP64 fault, patches of at most "
                     "128x128, static nested bands around the nucleation (no tagging)",
           "execution": "CUDA graph of 2 subcycled coarse steps (tmk_amr_graph_create), replayed",
           "tuning": {"autotuned": bool(autotune), "per_level": tunings},
           "device_status": status}
    graph.close()
    h.close()
    for lv in levels:
        lv.close()
    ctx.close()
    return out


def rupture_errors(make_scenario, nsteps, offsets_km, stream, graph_steps=0):
    """The mixed form against the plain FP64 form (the oracle-pinned one) on the
    same level from the same initial state: both run `nsteps` steps with fault
    stations at the nucleation centre +- offsets_km; returns the largest
    relative errors of arrival time, final slip and peak slip rate at the
    stations, the volume particle-velocity error, the friction solves that hit
    the bracket edge or the iteration limit in each form (status info[2]), and
    the mixed form's rate when `graph_steps` > 0 (steps replayed from a graph)."""
    import numpy as np
    import torch
    from tetemoko_gb300 import _capi as A, rupture as R
    from tetemoko_gb300.level import Context, LinElastLevelGodunov
    from tetemoko_gb300.stations import Stations
    res = {}
    for prec in (A.TMK_PREC_FP64, A.TMK_PREC_MIXED):
        sc = make_scenario(prec)
        ctx = Context(sc)
        lvl = LinElastLevelGodunov(ctx, [(0, 0, sc.nx - 1, sc.ny - 1)])
        lvl.set_patch(0, sc.initial_U(), sc.initial_B())
        xc = sc.nx * sc.dx / 2.0
        fx = [xc + s * d for d in offsets_km for s in (-1.0, 1.0)]
        st = Stations(lvl, fx, [], capacity=1024)
        st.attach()
        dt, t = sc.dt(), 0.0
        chunks = []
        for n in range(nsteps):
            lvl.step(t, dt, stream)
            t += dt
            if (n + 1) % 1000 == 0 or n + 1 == nsteps:
                torch.cuda.synchronize()
                chunks.append(st.read())
        rec = {"time": np.concatenate([c["time"] for c in chunks]),
               "fault": np.concatenate([c["fault"] for c in chunks])}
        law = sc.scheme.fault_law
        thr = sc.rs.rupture_threshold if law == A.TMK_FAULT_RS else sc.sw.rupture_threshold
        U, _ = lvl.get_patch(0)
        rc, info = lvl.status()
        res[prec] = (R.station_metrics(rec, law, thr), U, rc, info)
        st.close()
        rate = None
        if prec == A.TMK_PREC_MIXED and graph_steps:
            graph = lvl.graph(graph_steps, t, dt)
            graph.launch(t, stream)
            t += graph_steps * dt
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            nrep = max(1, nsteps // graph_steps)
            e0.record(stream)
            for _ in range(nrep):
                graph.launch(t, stream)
                t += graph_steps * dt
            e1.record(stream)
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / (nrep * graph_steps)
            rate = {"value": sc.nx * sc.ny / (ms * 1e-3), "unit": UNIT, "ms_per_step": ms,
                    "steps": nrep * graph_steps,
                    "execution": f"CUDA graph of {graph_steps} level steps, replayed (after the error run)"}
            graph.close()
        res["rate"] = rate
        lvl.close()
        ctx.close()
    m64, U64, rc64, info64 = res[A.TMK_PREC_FP64]
    mm, Um, rcm, infom = res[A.TMK_PREC_MIXED]
    out = R.compare(mm, m64)
    out["volume_velocity"] = R.velocity_error(Um, U64)
    out["bounds"] = {"arrival": 5e-3, "final_slip": 1e-3}
    out["within_bounds"] = bool(out["arrival"] is not None and out["arrival"] < 5e-3 and out["final_slip"] < 1e-3)
    out["steps"] = nsteps
    out["stations_km_from_nucleation"] = [s * d for d in offsets_km for s in (-1, 1)]
    out["bracket_limited_solves"] = {"fp64": info64[2], "mixed": infom[2]}
    out["status"] = {"fp64": rc64, "mixed": rcm}
    out["reference"] = "the plain FP64 GPU form (equal to the FP64 oracle to 1e-11 per step), same initial state"
    return out, res["rate"]


def amr3_measurement(coarse_steps, stream, regrid_interval=2):
    """Three levels at ratio 4 over the slip-weakening 512x256 base (dx 0.1 km,
    finest 6.25 m) with Drucker-Prager plasticity (1 MPa cohesion, background
    normal stresses from plas_Psi = 30 degrees), refined by device tags on the
    fault row's slip rate (>= 1e-3 m/s) and on velocity gradients, regridded
    every `regrid_interval` coarse steps with boxes of 8 to 64 cells
    (blocking factor 8, maximum 64, Berger-Rigoutsos on the host), mixed form.
    The subcycled steps are timed with CUDA events; each regrid (tags, boxes,
    new levels, prolongation, copy) by the host clock, reported apart."""
    import torch
    from tetemoko_gb300 import _capi as A, scenarios as S
    from tetemoko_gb300.amr import AMRHierarchy, regrid
    from tetemoko_gb300.level import Context, LinElastLevelGodunov
    sc = S.slip_weakening(nx=512, ny=256, precision=A.TMK_PREC_MIXED, plasticity=True, cohesion=1.0, plas_psi=30)
    ctx = Context(sc)
    ratios = [4, 4]
    base = LinElastLevelGodunov(ctx, tile_boxes(0, 0, sc.nx - 1, sc.ny - 1, 64))
    base.set_level(sc.initial_U(), sc.initial_B())
    box_args = dict(block_factor=8, max_grid_size=64, fill_ratio=0.7)

    def tps(initial):
        return [A.tag_params(level=l, initial=initial, refine_thresh=0.01, tag_buffer=2, slip_rate_thresh=1e-3)
                for l in range(2)]

    # the initial hierarchy from tagCellsInit's nucleation marks
    t0 = time.perf_counter()
    levels = regrid([base], ratios, tps(True), max_level=2, stream=stream, **box_args)
    torch.cuda.synchronize()
    init_s = time.perf_counter() - t0
    dt0 = sc.dt()
    t = 0.0
    step_ms, regrid_s, updates, nregrid = 0.0, 0.0, 0, 0
    sizes = set()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    done = 0
    while done < coarse_steps:
        h = AMRHierarchy(levels, ratios[:len(levels) - 1], time=t)
        n = min(regrid_interval, coarse_steps - done)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(n):
            h.step(dt0, stream)
        e1.record(stream)
        torch.cuda.synchronize()
        step_ms += e0.elapsed_time(e1)
        updates += h.cell_updates() * n
        t = h.time(0)
        h.close()
        done += n
        if done < coarse_steps:
            r0 = time.perf_counter()
            old = levels
            levels = regrid(levels, ratios, tps(False), stream=stream, **box_args)
            torch.cuda.synchronize()
            regrid_s += time.perf_counter() - r0
            nregrid += 1
            for lv in old[1:]:
                if all(lv is not nl for nl in levels):
                    lv.close()
        for lv in levels[1:]:
            for b in lv.boxes:
                sizes.add(max(b[2] - b[0] + 1, b[3] - b[1] + 1))
    status = [lv.status()[1] for lv in levels]
    cells = [sum((b[2] - b[0] + 1) * (b[3] - b[1] + 1) for b in lv.boxes) for lv in levels]
    out = {"value": updates / (step_ms * 1e-3), "unit": "cell-updates/s",
           "ms_per_coarse_step": step_ms / coarse_steps, "coarse_steps": coarse_steps,
           "regrids": nregrid, "regrid_ms_each": 1e3 * regrid_s / max(1, nregrid),
           "initial_hierarchy_ms": 1e3 * init_s,
           "cells_per_level_at_end": cells, "patches_per_level_at_end": [len(lv.boxes) for lv in levels],
           "patch_side_range": [min(sizes), max(sizes)] if sizes else None,
           "config": "3 levels, ratio 4, base 512x256 at dx=0.1 km (finest 6.25 m), slip weakening (mu_s 0.677, "
                     "mu_d 0.525, Dc 0.4 m, side 2 at offset 11), Drucker-Prager plasticity with 1 MPa cohesion "
                     "(b = c cos(phi), an extension), background from plas_Psi = 30 deg, tags: fault-row slip rate "
                     ">= 1e-3 m/s (an extension) or velocity gradient >= 0.01, tag buffer 2, boxes: blocking "
                     "factor 8, max 64, fill ratio 0.7, regrid every 2 coarse steps, FP32 volume / FP64 fault",
           "execution": "tmk_amr_step per coarse step (levels change every regrid); regrid on the device (tags, "
                        "prolongation, copy) with host box generation",
           "device_status": status}
    for lv in levels:
        lv.close()
    ctx.close()
    return out


ENSEMBLE_SIZE = 64


def ensemble_measurement(steps, warmup, stream, nscen=ENSEMBLE_SIZE, autotune=True, max_grid=1024):
    """64 independent rate-and-state scenarios (seeded friction, lognormal shear
    prestress, grids drawn from 256x128 / 512x256 / 1024x512) stepped as one
    level in the mixed form; steps replayed from a CUDA graph.  Returns the JSON
    object of the measurement."""
    import torch
    from tetemoko_gb300 import _capi as A, scenarios as S
    from tetemoko_gb300.level import Context, LinElastEnsemble
    members = [S.ensemble_member(k, precision=A.TMK_PREC_MIXED) for k in range(nscen)]
    ctxs = [Context(sc) for sc, _ in members]
    doms = [(0, 0, sc.nx - 1, sc.ny - 1) for sc, _ in members]
    ens = LinElastEnsemble(ctxs, doms, [tile_boxes(0, 0, sc.nx - 1, sc.ny - 1, max_grid) for sc, _ in members])
    for k, (sc, tau0) in enumerate(members):
        U, B = S.prestressed_state(sc, tau0)
        ens.set_scenario(k, U, B)
    dt = members[0][0].dt()
    tuning = ens.autotune(0.0, dt, steps=4, stream=stream)[0].as_dict() if autotune else None
    t = 0.0
    for _ in range(warmup):
        ens.step(t, dt, stream)
        t += dt
    gsteps = 20
    graph = ens.graph(gsteps, t, dt)
    graph.launch(t, stream)
    t += gsteps * dt
    torch.cuda.synchronize()
    nrep = max(1, steps // gsteps)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(nrep):
        graph.launch(t, stream)
        t += gsteps * dt
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    # per-kernel times: a few steps call by call with events around each launch
    # (the fault kernel then runs before the marching kernels, not beside them)
    nprof = 10
    ens.profile(True, nprof)
    for _ in range(nprof):
        ens.step(t, dt, stream)
        t += dt
    torch.cuda.synchronize()
    prof, _ = ens.profile_read()
    ens.profile(False)
    cells = ens.cells()
    grids = {}
    for sc, _ in members:
        grids[f"{sc.nx}x{sc.ny}"] = grids.get(f"{sc.nx}x{sc.ny}", 0) + 1
    out = {"value": cells * gsteps * nrep / (ms * 1e-3), "unit": "cell-updates/s",
           "ms_per_step": ms / (gsteps * nrep), "steps": gsteps * nrep, "scenarios": nscen,
           "cells": cells, "patches": len(ens.boxes), "grids": grids,
           "launches_per_step": ens.launches_per_step(),
           "kernel_ms": {"exchange": prof[0], "fault": prof[1], "volume": prof[2], "step_serialised": prof[3]},
           "volume_hbm_gbs": BYTES_PER_CELL_MIXED * cells / (prof[2] * 1e-3) / 1e9,
           "config": "rate-and-state aging law, a ~ U[0.006,0.012], b-a ~ U[0.002,0.006], L ~ U[0.01,0.05] m "
                     "(seed 5000+k), shear prestress 70 exp(g - s^2/2) MPa with g Gaussian, exponential "
                     "covariance, 1 km correlation, s = 0.1 (seed 6000+k), dx = 0.1 km, FP32 volume / FP64 "
                     f"fault, patches of at most {max_grid}x{max_grid}, one level of all scenarios",
           "execution": f"CUDA graph of {gsteps} ensemble steps (tmk_ensemble_create + tmk_level_graph_create), "
                        "replayed",
           "tuning": {"autotuned": bool(autotune), "choice": tuning},
           "device_status": ens.status()[1]}
    graph.close()
    ens.close()
    for c in ctxs:
        c.close()
    return out


THREE_D = (192, 96, 96)
# algorithmic bytes per cell of the 3-D step: the 18 evolving FP64 components
# of the state read and written once (lambda and gamma carry no flux)
BYTES_PER_CELL_3D = 18 * 8 * 2


def three_d_measurement(steps, warmup, stream, fp64_steps=3, cpu_seconds=5.0, size=THREE_D):
    """One 192x96x96 patch of the rate-and-state workload in 3-D (a
    CH_SPACEDIM == 3 build: the 3-D corner transport upwind step, the fault the
    y-lo plane), stepped through tmk_patch_update_state_3d in the mixed form
    and in the plain FP64 form; the oracle's 3-D step on a 24x12x12 patch for
    the CPU rate.  Returns the JSON object of the measurement."""
    import torch
    import numpy as np
    from tetemoko_gb300 import _capi as A, scenarios as S
    from tetemoko_gb300.level import Context, LinElastLevelGodunov3D, LinElastPatchGodunov3D
    nx, ny, nz = size
    g = A.TMK_NGHOST
    lo, hi = (0, 0, 0), (nx - 1, ny - 1, nz - 1)

    def state(sc):
        rng = np.random.default_rng(2024)
        U = np.empty((22, nz + 2 * g, ny + 2 * g, nx + 2 * g))
        U[:] = sc.background()[:, None, None, None]
        U[[0, 11]] += 1e-3 * rng.standard_normal((2,) + U.shape[1:])
        B1 = sc.initial_B(xlo=0, xhi=nx - 1)
        B = np.ascontiguousarray(np.repeat(B1[:, None, :], nz + 2 * g, axis=1))
        return U, B

    out = {}
    for prec, n in ((A.TMK_PREC_MIXED, steps), (A.TMK_PREC_FP64, fp64_steps)):
        sc = S.rate_state(nx=nx, ny=ny, dx=0.1, precision=prec)
        ctx = Context(sc)
        pg = LinElastPatchGodunov3D(ctx, (lo, hi))
        pg.set_current_box((lo, hi))
        U0, B0 = state(sc)
        Ud = torch.from_numpy(U0).cuda()
        Bd = torch.from_numpy(B0).cuda()
        dt = sc.dt() / 3 ** 0.5      # the 3-D CFL bound
        t = 0.0
        for _ in range(warmup):
            pg.set_current_time(t)
            pg.update_state(Ud, (-g, -g, -g), dt, B=Bd, blo=(-g, -g), stream=stream)
            t += dt
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(n):
            pg.set_current_time(t)
            pg.update_state(Ud, (-g, -g, -g), dt, B=Bd, blo=(-g, -g), stream=stream)
            t += dt
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / n
        out[prec] = {"value": nx * ny * nz / (ms * 1e-3), "unit": UNIT, "ms_per_step": ms, "steps": n,
                     "finite": bool(torch.isfinite(Ud).all().item())}
        ctx.close()
    mixed, fp64 = out[A.TMK_PREC_MIXED], out[A.TMK_PREC_FP64]
    # the same domain as Chombo-sized patches of 32^3: one call per patch, and
    # the level's patch loop in one batched call (mixed form)
    tiles = {}
    tsz = 32
    if nx % tsz == 0 and ny % tsz == 0 and nz % tsz == 0:
        sc = S.rate_state(nx=nx, ny=ny, dx=0.1, precision=A.TMK_PREC_MIXED)
        ctx = Context(sc)
        pg = LinElastPatchGodunov3D(ctx, (lo, hi))
        U0, B0 = state(sc)
        patches = []
        for k0 in range(0, nz, tsz):
            for j0 in range(0, ny, tsz):
                for i0 in range(0, nx, tsz):
                    v = ((i0, j0, k0), (i0 + tsz - 1, j0 + tsz - 1, k0 + tsz - 1))
                    U = torch.from_numpy(np.ascontiguousarray(
                        U0[:, k0:k0 + tsz + 2 * g, j0:j0 + tsz + 2 * g, i0:i0 + tsz + 2 * g])).cuda()
                    B = None
                    if j0 == 0:
                        B = torch.from_numpy(np.ascontiguousarray(B0[:, k0:k0 + tsz + 2 * g, i0:i0 + tsz + 2 * g])).cuda()
                    patches.append((v, U, (i0 - g, j0 - g, k0 - g), B, (i0 - g, k0 - g)))
        dt = sc.dt() / 3 ** 0.5

        def per_patch(t):
            pg.set_current_time(t)
            for v, U, ulo, B, blo in patches:
                pg.set_current_box(v)
                pg.update_state(U, ulo, dt, B=B, blo=blo, stream=stream)

        def batched(t):
            pg.set_current_time(t)
            pg.update_states(patches, dt, stream=stream)

        # the device level over the same patches: its step exchanges the
        # ghost cells on the device before the batched patch loop
        lvl = LinElastLevelGodunov3D(ctx, [v for v, *_ in patches], (lo, hi))
        for p, (v, U, ulo, B, blo) in enumerate(patches):
            lvl.set_patch(p, U, B)

        def level_step(t):
            lvl.step(t, dt, stream)

        def level_exchange(t):
            lvl.exchange(stream)

        def run(fn):
            t = 0.0
            for _ in range(warmup):
                fn(t)
                t += dt
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(steps):
                fn(t)
                t += dt
            e1.record(stream)
            torch.cuda.synchronize()
            return e0.elapsed_time(e1) / steps

        for name, fn in (("per_patch_calls", per_patch), ("batched", batched), ("level", level_step)):
            ms = run(fn)
            tiles[name] = {"value": nx * ny * nz / (ms * 1e-3), "unit": UNIT, "ms_per_step": ms}
        tiles["level"]["exchange_ms"] = run(level_exchange)
        tiles["level"]["note"] = ("tmk_level3d_step: the ghost exchange between the patches on the device, then the "
                                  "batched patch loop")
        tiles["patches"] = len(patches)
        tiles["patch"] = f"{tsz}^3 (per_patch_calls and batched: ghost exchange left out, the caller's)"
        lvl.close()
        ctx.close()
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except Exception:
        pass
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    achieved = BYTES_PER_CELL_3D * nx * ny * nz / (mixed["ms_per_step"] * 1e-3) / 1e9
    traffic = None
    tf = os.path.join(ROOT, "profiles", "patch_step_3d_mixed_192x96x96.traffic.json")
    if os.path.exists(tf):
        try:
            # measured per cell on a 128x64x64 patch; every pass is a pass over the patch
            traffic = json.load(open(tf))["bytes_per_cell"] * nx * ny * nz
        except Exception:
            traffic = None
    cpu = None
    if cpu_seconds > 0:
        import oracle as O
        sc = S.rate_state(nx=24, ny=12, dx=0.1)
        cn = (24, 12, 12)
        U = np.empty((22, cn[2] + 2 * g, cn[1] + 2 * g, cn[0] + 2 * g))
        U[:] = sc.background()[:, None, None, None]
        B = np.ascontiguousarray(np.repeat(sc.initial_B(xlo=0, xhi=cn[0] - 1)[:, None, :], cn[2] + 2 * g, axis=1))
        dt = sc.dt() / 3 ** 0.5
        n, t0 = 0, time.perf_counter()
        while time.perf_counter() - t0 < cpu_seconds or n == 0:
            O.patch_update_state_3d(sc, U, (-g, -g, -g), (0, 0, 0), (cn[0] - 1, cn[1] - 1, cn[2] - 1), (0, 0, 0),
                                    (cn[0] - 1, cn[1] - 1, cn[2] - 1), B, (-g, -g), sc.dx, n * dt, dt)
            n += 1
        el = time.perf_counter() - t0
        cpu = {"value": cn[0] * cn[1] * cn[2] * n / el, "unit": UNIT, "cores": 1, "kind": "port",
               "sample": f"{n} oracle 3-D patch steps of a 24x12x12 patch (the same scenario), one thread"}
    return {"workload": f"rate-and-state fault plane y=0, one {nx}x{ny}x{nz} patch, dx = 0.1 km, PPM + "
                        "primitive limiting, dt = CFL 0.9/sqrt(3)",
            "value": mixed["value"], "unit": UNIT, "ms_per_step": mixed["ms_per_step"], "steps": mixed["steps"],
            "form": "mixed (FP32 volume arithmetic and intermediates, FP64 state, friction and boundary data)",
            "fp64_plain": fp64, "mixed_over_fp64": mixed["value"] / fp64["value"],
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                         "frac": achieved / hbm_peak, "traffic": traffic,
                         "algorithmic_bytes_per_step": BYTES_PER_CELL_3D * nx * ny * nz,
                         "kernel": "the whole 3-D step (18 launches: FP32 copy, 3 predictors, 4 first-pass, "
                                   "3 paired second-pass + 1 fault-plane and 4 final face passes, update, "
                                   "boundary data)",
                         "timing": f"CUDA events on the launch stream around {mixed['steps']} steps"},
            "cpu_baseline": cpu,
            "patches_32": tiles,
            "finite": mixed["finite"] and fp64["finite"],
            "execution": "one tmk_patch_update_state_3d call per step, device FABs"}


def host_threads():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def run_reference(args):
    rank, world, _ = rank_env()
    if rank != 0:
        return 0
    from tetemoko_gb300 import scenarios as S
    nthreads = host_threads()
    nx, ny = args.nx, args.ny
    sc = S.rate_state(nx=nx, ny=ny)
    # size the per-step sample so that warm-up + steps stay within about two minutes
    probe_rate, _ = cpu_sample(sc, min(2.0, args.cpu_seconds), nthreads, strip_rows=min(64, ny))
    budget = 120.0
    steps = max(1, args.steps) + max(0, args.warmup)
    rows = int(probe_rate * budget / steps / nx)
    rows = max(min(16, ny), min(ny, (rows // 8) * 8))
    import oracle as O
    sub = S.rate_state(nx=nx, ny=rows, dx=sc.dx)
    boxes = O.tile_boxes(sub.nx, sub.ny, 128)
    U, B = sub.initial_U(), sub.initial_B()
    dt, t = sub.dt(), 0.0
    for _ in range(args.warmup):
        O.level_step(sub, U, B, boxes, t, dt, nthreads=nthreads)
        t += dt
    t0 = time.perf_counter()
    for _ in range(args.steps):
        O.level_step(sub, U, B, boxes, t, dt, nthreads=nthreads)
        t += dt
    el = time.perf_counter() - t0
    value = sub.nx * sub.ny * args.steps / el
    sample = (f"each step: one level step of a {nx}x{rows} strip (fault row included) of the {nx}x{ny} "
              f"workload, 128x128 patches, OpenMP over patches")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": workload_config(nx, ny),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthreads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference's Chombo/Fortran build cannot be compiled here (no Fortran compiler, no "
                "Chombo); its path is timed through the FP64 C++ oracle that restates it",
    }
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=4000)    # the workload's max_step
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--fp64-steps", type=int, default=20)
    ap.add_argument("--fp64-kernel", default="march", choices=["march", "tile"])
    ap.add_argument("--e2e-steps", type=int, default=10)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--amr-steps", type=int, default=16)   # timed coarse steps of the AMR measurement
    ap.add_argument("--amr-only", action="store_true")      # only the AMR measurement (profiling runs)
    ap.add_argument("--ensemble-steps", type=int, default=200)   # timed steps of the ensemble measurement
    ap.add_argument("--ensemble-only", action="store_true")
    ap.add_argument("--ensemble-max-grid", type=int, default=1024)  # largest patch side (1024: one patch per scenario)
    ap.add_argument("--no-autotune", dest="autotune", action="store_false")   # keep the default tuning
    ap.add_argument("--three-d-steps", type=int, default=20)   # timed steps of the 3-D measurement
    ap.add_argument("--three-d-only", action="store_true")
    ap.add_argument("--three-d-size", default="192x96x96")   # profiling runs use a smaller patch
    ap.add_argument("--error-steps", type=int, default=4000)   # mixed vs FP64 rupture errors (max_step)
    ap.add_argument("--sw-steps", type=int, default=1000)      # slip-weakening 512x256 level (its max_step)
    ap.add_argument("--amr3-steps", type=int, default=100)     # coarse steps of the regridded 3-level ratio-4 run
    ap.add_argument("--amr3-only", action="store_true")
    ap.add_argument("--nx", type=int, default=NX)
    ap.add_argument("--ny", type=int, default=NY)
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        return run_reference(args)

    import numpy as np
    import torch
    import torch.distributed as dist

    from tetemoko_gb300 import _capi as A, scenarios as S
    from tetemoko_gb300.level import Context, LinElastLevelGodunov

    rank, world, local = rank_env()
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if world > 1:
            dist.barrier()

    nx, ny = args.nx, args.ny
    cells = nx * ny
    stream = torch.cuda.current_stream()

    def make_level(prec, volume_kernel=A.TMK_VOLUME_AUTO):
        sc = S.rate_state(nx=nx, ny=ny, precision=prec)
        sc.scheme.volume_kernel = volume_kernel
        ctx = Context(sc)
        lvl = LinElastLevelGodunov(ctx, [(0, 0, nx - 1, ny - 1)])
        lvl.set_patch(0, sc.initial_U(), sc.initial_B())
        return sc, ctx, lvl

    def timed(lvl, sc, steps, warmup, profile=False, sampler=None, graph_steps=0):
        dt = sc.dt()
        t = 0.0
        for _ in range(warmup):
            lvl.step(t, dt, stream)
            t += dt
        graph = None
        if graph_steps:
            # record graph_steps steps once; the timed loop replays them
            graph = lvl.graph(graph_steps, t, dt)
            for _ in range(2):
                graph.launch(t, stream)
                t += graph_steps * dt
        if profile:
            lvl.profile(True, steps)
        torch.cuda.synchronize()
        barrier()
        torch.cuda.synchronize()
        if sampler:
            sampler.start()
            if isinstance(sampler, ClockSampler):
                time.sleep(0.4)     # nvidia-smi's first sample
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        if graph is not None:
            for _ in range(steps // graph_steps):
                graph.launch(t, stream)
                t += graph_steps * dt
        else:
            for _ in range(steps):
                lvl.step(t, dt, stream)
                t += dt
        e1.record(stream)
        torch.cuda.synchronize()
        clocks = sampler.stop() if sampler else None
        barrier()
        ms = e0.elapsed_time(e1)
        prof = lvl.profile_read() if profile else None
        if profile:
            lvl.profile(False)
        rc, info = lvl.status()
        if graph is not None:
            graph.close()
        return ms, prof, clocks, (rc, info)

    # ---- mixed form (headline): an uninstrumented timed pass for the value, then
    # a second timed pass with CUDA events around every launch for the roofline
    # (events between the fault and volume kernels serialise their overlap)
    if args.amr_only:
        amr = amr_measurement(args.amr_steps, args.warmup, stream, args.autotune)
        if rank == 0:
            print(json.dumps({"amr": amr}), flush=True)
        return 0
    if args.three_d_only:
        td = three_d_measurement(args.three_d_steps, 3, stream, cpu_seconds=0.0,
                                 size=tuple(int(v) for v in args.three_d_size.split("x")))
        if rank == 0:
            print(json.dumps({"three_d": td}), flush=True)
        return 0
    if args.amr3_only:
        a3 = amr3_measurement(args.amr3_steps, stream)
        if rank == 0:
            print(json.dumps({"amr3": a3}), flush=True)
        return 0
    if args.ensemble_only:
        ens = ensemble_measurement(args.ensemble_steps, args.warmup, stream, autotune=args.autotune,
                                   max_grid=args.ensemble_max_grid)
        if rank == 0:
            print(json.dumps({"ensemble": ens}), flush=True)
        return 0
    sc, ctx, lvl = make_level(A.TMK_PREC_MIXED)
    # work-list shape and fault-kernel variant picked by the autotuner (trial
    # steps from the initial state, which it puts back)
    tuning, tune_ms = None, None
    if args.autotune:
        t, tune_ms = lvl.autotune(0.0, sc.dt(), steps=10, stream=stream)
        tuning = t.as_dict()
    # steps replayed from a CUDA graph of graph_steps recorded steps (the
    # largest even divisor of --steps up to 100); also timed call by call
    graph_steps = next((g for g in range(min(100, args.steps), 1, -1) if args.steps % g == 0 and g % 2 == 0), 0)
    _, ctx_c, lvl_c = make_level(A.TMK_PREC_MIXED)       # same workload from its initial state
    if args.autotune:
        lvl_c.set_tuning(lvl.tuning())
    ms_call, _, _, _ = timed(lvl_c, sc, args.steps, args.warmup, profile=False)
    value_call, _ = replica_rate(cells, args.steps, ms_call * 1e-3, world, device="cuda")
    lvl_c.close()
    ctx_c.close()
    sampler = make_clock_sampler() if rank == 0 else None
    ms, _, clocks, st = timed(lvl, sc, args.steps, args.warmup, profile=False, sampler=sampler,
                              graph_steps=graph_steps)
    value, secs = replica_rate(cells, args.steps, ms * 1e-3, world, device="cuda")
    ms = secs * 1e3
    launches = lvl.launches_per_step() * args.steps
    nprof_steps = min(args.steps, 200)
    _, prof, _, _ = timed(lvl, sc, nprof_steps, 1, profile=True)
    (ex_ms, fault_ms, vol_ms, step_ms), nprof = prof
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except Exception:
        pass
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    achieved = BYTES_PER_CELL_MIXED * cells / (vol_ms * 1e-3) / 1e9
    traffic = None
    tf = os.path.join(ROOT, "profiles", "volume_kernel_mixed_2048x1024.traffic.json")
    if os.path.exists(tf):
        try:
            traffic = json.load(open(tf)).get("dram_bytes_per_launch")
        except Exception:
            traffic = None
    roofline = {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                "frac": achieved / hbm_peak, "traffic": traffic,
                "kernel": "volume update: march_kernel<float,0> (in-plane) + march_kernel<float,1> (antiplane)",
                "algorithmic_bytes_per_launch": BYTES_PER_CELL_MIXED * cells, "peak_source": peak_src,
                "kernel_ms": vol_ms, "fault_kernel_ms": fault_ms, "step_ms_profiled": step_ms,
                "timing": f"average over a second timed pass of {nprof} steps with CUDA events on the launch "
                          "stream around each launch (serialises the fault/volume overlap of the headline pass)"}

    # ---- e2e through the C ABI with pinned host buffers: the state lives in a
    # host FAB (as a Chombo FArrayBox does); each step copies in what the step
    # reads and copies out what it rewrites (tmk_level_put_valid / take_valid:
    # the 18 evolving components of the valid cells, and the fault data)
    ushape, bshape = lvl.patch_shapes(0)
    Uh = torch.empty(ushape, dtype=torch.float64).pin_memory()
    Bh = torch.empty(bshape, dtype=torch.float64).pin_memory()
    lvl.get_patch(0, Uh.numpy(), Bh.numpy())
    dt = sc.dt()
    t = 0.0
    for _ in range(2):
        lvl.put_valid(0, Uh.numpy(), Bh.numpy())
        lvl.step(t, dt, stream)
        lvl.take_valid(0, Uh.numpy(), Bh.numpy())
        t += dt
    torch.cuda.synchronize()
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.e2e_steps):
        lvl.put_valid(0, Uh.numpy(), Bh.numpy())
        lvl.step(t, dt, stream)
        lvl.take_valid(0, Uh.numpy(), Bh.numpy())
        t += dt
    torch.cuda.synchronize()
    e2e_value, _ = replica_rate(cells, args.e2e_steps, time.perf_counter() - t0, world, device="cuda")
    h2d = 18 * cells * 8 + Bh.numel() * 8
    lvl.close()
    ctx.close()

    # ---- plain FP64 form on the same workload
    fp64_kernel = {"march": A.TMK_VOLUME_MARCH, "tile": A.TMK_VOLUME_TILE}[args.fp64_kernel]
    sc64, ctx64, lvl64 = make_level(A.TMK_PREC_FP64, fp64_kernel)
    n64 = max(1, args.fp64_steps)
    ms64, prof64, _, st64 = timed(lvl64, sc64, n64, 3, profile=True)
    value64, secs64 = replica_rate(cells, n64, ms64 * 1e-3, world, device="cuda")
    ms64 = secs64 * 1e3
    vol64 = prof64[0][2]
    lvl64.close()
    ctx64.close()

    # ---- the slip error of the mixed form at the benchmarked configuration
    errors = None
    if args.error_steps > 0:
        errors, _ = rupture_errors(lambda p: S.rate_state(nx=nx, ny=ny, precision=p), args.error_steps,
                                   (5.0, 10.0, 20.0, 40.0, 60.0, 80.0), stream)
    # ---- the slip-weakening 512x256 level (the CPU-runnable workload), mixed
    # form rate and its rupture errors against the FP64 form
    sw_level = None
    if args.sw_steps > 0:
        sw_err, sw_rate = rupture_errors(lambda p: S.slip_weakening(nx=512, ny=256, precision=p), args.sw_steps,
                                         (3.0, 6.0, 9.0, 12.0, 15.0, 20.0), stream, graph_steps=100)
        sw_level = dict(sw_rate or {})
        sw_level["config"] = ("slip-weakening planar fault, uniform 512x256, dx=0.1 km, mu_s=0.677, mu_d=0.525, "
                              "Dc=0.4 m, 120 MPa normal / 70 MPa shear, 3 km nucleation window at 81.6 MPa, "
                              "side-2 components at offset 11, FP32 volume / FP64 fault")
        sw_level["errors"] = sw_err

    # ---- subcycled 4-level AMR hierarchy (rank 0 reports its own)
    amr = amr_measurement(args.amr_steps, 2, stream, args.autotune) if args.amr_steps > 0 else None
    # ---- 3 levels at ratio 4, slip weakening with plasticity, regridded every 2 coarse steps
    amr3 = amr3_measurement(args.amr3_steps, stream) if args.amr3_steps > 0 else None
    # ---- ensemble of 64 independent scenarios in one level
    ens = ensemble_measurement(args.ensemble_steps, 3, stream, autotune=args.autotune, max_grid=args.ensemble_max_grid) \
        if args.ensemble_steps > 0 else None

    # ---- the 3-D patch step
    three_d = three_d_measurement(args.three_d_steps, 3, stream, cpu_seconds=min(5.0, args.cpu_seconds)) \
        if args.three_d_steps > 0 and rank == 0 else None

    # ---- CPU baseline (rank 0, N = 1 only)
    cpu = None
    if rank == 0 and world == 1 and args.cpu_seconds > 0:
        nthreads = host_threads()
        rate, desc = cpu_sample(S.rate_state(nx=nx, ny=ny), args.cpu_seconds, nthreads, strip_rows=min(ny, 256))
        cpu = {"value": rate, "unit": UNIT, "cores": nthreads, "kind": "port", "sample": desc}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
            "config": workload_config(nx, ny),
            "roofline": roofline,
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": h2d,
                    "note": "state in a pinned host FP64 FAB; per step: tmk_level_put_valid (the 18 evolving "
                            "components of the valid cells and the fault data, host->device), level step, "
                            "tmk_level_take_valid (the same, device->host)"},
            "gpu_launches": launches,
            "clocks": clocks,
            "execution": (f"steps replayed from a CUDA graph of {graph_steps} recorded level steps "
                          "(tmk_level_graph_create / tmk_graph_launch)") if graph_steps else "one call per step",
            "tuning": {"autotuned": bool(args.autotune), "choice": tuning, "trial_ms_per_step": tune_ms},
            "per_call": {"value": value_call, "unit": UNIT, "ms_per_step": ms_call / args.steps,
                         "note": "the same steps, one tmk_level_step call each"},
            "sw_level": sw_level,
            "amr": amr,
            "amr3": amr3,
            "ensemble": ens,
            "three_d": three_d,
            # the two forms side by side and the mixed form's errors last, where
            # the end of a truncated log still shows them
            "device_status": {"mixed": st[1], "fp64": st64[1]},
            "fp64_plain": {"value": value64, "unit": UNIT, "ms_per_step": ms64 / n64, "steps": n64,
                           "volume_kernel": args.fp64_kernel, "volume_kernel_ms": vol64,
                           "volume_hbm_gbs": BYTES_PER_CELL_FP64 * cells / (vol64 * 1e-3) / 1e9},
            "mixed_over_fp64": value / value64,
            "errors": errors,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
