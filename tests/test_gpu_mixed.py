"""Mixed form (FP32 volume, FP64 friction) against the FP64 oracle on a rupture.

Metrics at fault stations 3-9 km either side of the nucleation centre:
  * rupture-front arrival time: first crossing of V = 1e-3 m/s, interpolated
    linearly between steps; tolerance 0.5 % relative;
  * final slip (slip total after the run); tolerance 1e-3 relative;
  * peak slip rate over the run; tolerance 1e-2 relative;
and the largest particle-velocity difference in the volume, relative to the
largest FP64 particle velocity; tolerance 1e-2.
"""
import numpy as np
import pytest

import oracle as O
from tetemoko_gb300 import _capi as A, scenarios as S

pytestmark = pytest.mark.gpu

NSTEPS = 300
ARRIVAL_RTOL = 5e-3
SLIP_RTOL = 1e-3
PEAK_RTOL = 1e-2
VEL_RTOL = 1e-2


def _stations(sc):
    x0 = sc.rs.x0
    xs = [x0 + s * d for d in (3.0, 5.0, 7.0, 9.0) for s in (-1, 1)]
    return [int(round(x / sc.dx - 0.5)) for x in xs]


def _arrival(ts, V, thr):
    """linear-in-time crossing of thr by the slip-rate history V (per station)."""
    out = []
    for k in range(V.shape[1]):
        v = V[:, k]
        idx = np.nonzero(v > thr)[0]
        if len(idx) == 0:
            out.append(np.nan)
            continue
        n = idx[0]
        if n == 0:
            out.append(ts[0])
            continue
        a = (thr - v[n - 1]) / (v[n] - v[n - 1])
        out.append(ts[n - 1] + a * (ts[n] - ts[n - 1]))
    return np.array(out)


def _run_gpu(sc, st):
    from tetemoko_gb300.level import Context, LinElastLevelGodunov
    ctx = Context(sc)
    lvl = LinElastLevelGodunov(ctx, [(0, 0, sc.nx - 1, sc.ny - 1)])
    lvl.set_patch(0, sc.initial_U(), sc.initial_B())
    dt, t = sc.dt(), 0.0
    g = A.TMK_NGHOST
    Vh, ts = [], []
    for _ in range(NSTEPS):
        lvl.step(t, dt)
        t += dt
        _, B = lvl.get_patch(0)
        Vh.append(B[2, [i + g for i in st]].copy())
        ts.append(t)
    U, B = lvl.get_patch(0)
    rc, info = lvl.status()
    lvl.close()
    ctx.close()
    assert rc == 0, info
    return np.array(ts), np.array(Vh), U, B


def _run_oracle(sc, st):
    U, B = sc.initial_U(), sc.initial_B()
    dt, t = sc.dt(), 0.0
    g = A.TMK_NGHOST
    boxes = O.tile_boxes(sc.nx, sc.ny, 64)
    Vh, ts = [], []
    for _ in range(NSTEPS):
        assert O.level_step(sc, U, B, boxes, t, dt, nthreads=8) == 0
        t += dt
        Vh.append(B[2, [i + g for i in st]].copy())
        ts.append(t)
    return np.array(ts), np.array(Vh), U, B


def test_mixed_rupture_metrics_vs_fp64_oracle(cuda_lib):
    sc64 = S.rate_state(nx=256, ny=128, dx=0.1)
    scm = S.rate_state(nx=256, ny=128, dx=0.1, precision=A.TMK_PREC_MIXED)
    st = _stations(sc64)
    g = A.TMK_NGHOST
    tr, Vr, Ur, Br = _run_oracle(sc64, st)
    tm, Vm, Um, Bm = _run_gpu(scm, st)
    thr = sc64.rs.rupture_threshold
    ar, am = _arrival(tr, Vr, thr), _arrival(tm, Vm, thr)
    assert np.all(np.isfinite(ar)), "every station must rupture within the run"
    arr_err = np.max(np.abs(am - ar) / ar)
    slip_r, slip_m = Br[8, [i + g for i in st]], Bm[8, [i + g for i in st]]
    slip_err = np.max(np.abs(slip_m - slip_r) / np.abs(slip_r))
    peak_err = np.max(np.abs(Vm.max(axis=0) - Vr.max(axis=0)) / Vr.max(axis=0))
    vcomp = [0, 1, 2, 11, 12, 13]
    vs = (vcomp, slice(g, -g), slice(g, -g))
    vel_err = np.abs(Um[vs] - Ur[vs]).max() / np.abs(Ur[vs]).max()
    print(f"mixed vs FP64 oracle: arrival {arr_err:.2e}, final slip {slip_err:.2e}, "
          f"peak slip rate {peak_err:.2e}, volume velocity {vel_err:.2e}")
    assert arr_err < ARRIVAL_RTOL
    assert slip_err < SLIP_RTOL
    assert peak_err < PEAK_RTOL
    assert vel_err < VEL_RTOL


def test_fp64_level_equals_oracle_over_a_rupture(cuda_lib):
    """The plain FP64 form tracks the oracle through nucleation and rupture."""
    sc = S.rate_state(nx=256, ny=128, dx=0.1)
    st = _stations(sc)
    tr, Vr, Ur, Br = _run_oracle(sc, st)
    tg, Vg, Ug, Bg = _run_gpu(sc, st)
    g = A.TMK_NGHOST
    rel = np.abs(Ug - Ur)[:, g:-g, g:-g].max() / np.abs(Ur).max()
    relb = np.abs(Bg - Br)[:, g:-g].max(axis=1) / np.maximum(np.abs(Br[:, g:-g]).max(axis=1), 1e-300)
    print(f"FP64 GPU vs oracle after {NSTEPS} steps: U {rel:.2e}, B {relb.max():.2e}")
    assert rel < 1e-10
    assert relb.max() < 1e-10


@pytest.mark.parametrize("variant", ["slip_law", "slip_law_weakening", "per_face_aging"])
def test_mixed_fault_path_tracks_the_fp64_oracle(cuda_lib, variant):
    """The mixed form's latency-arranged rate-and-state path (per-face constants,
    reciprocal products, z-space Newton) on the laws and options the rupture run
    does not use: the slip law, its flash-weakening steady state, and per-face
    a, b, L.  Ten steps of a perturbed level against the FP64 oracle: the state
    to FP32 rounding of the volume (1e-4) and the fault data to 1e-3."""
    from tetemoko_gb300.level import Context, LinElastLevelGodunov
    from tests.helpers import perturbed_state, rel_err
    law = A.TMK_RS_AGING_LAW if variant == "per_face_aging" else A.TMK_RS_SLIP_LAW
    sc64 = S.rate_state(nx=64, ny=32, dx=0.1, state_law=law)
    scm = S.rate_state(nx=64, ny=32, dx=0.1, state_law=law, precision=A.TMK_PREC_MIXED)
    for sc in (sc64, scm):
        sc.rs.L = 0.5
        if variant == "slip_law_weakening":
            sc.rs.fexp, sc.rs.fw, sc.rs.Vw = 1.0, 0.2, 0.01
    F = S.friction_field(sc64, seed=4001) if variant == "per_face_aging" else None
    boxes = [(0, 0, 31, 15), (32, 0, 63, 15), (0, 16, 63, 31)]
    Ug = perturbed_state(sc64, np.random.default_rng(81), amp_v=0.05, amp_s=1.0)
    Bg = sc64.initial_B()
    Ur, Br = Ug.copy(), Bg.copy()
    ctx = Context(scm)
    lv = LinElastLevelGodunov(ctx, boxes)
    lv.set_level(Ug, Bg)
    if F is not None:
        lv.set_level_friction(F)
    dt = sc64.dt()
    for k in range(10):
        assert O.level_step(sc64, Ur, Br, boxes, k * dt, dt, fric=F) == 0
        lv.step(k * dt, dt)
    Um, Bm = Ug.copy(), Bg.copy()
    lv.get_level(Um, Bm)
    g = A.TMK_NGHOST
    assert lv.status()[0] == 0
    assert rel_err(Um[:, g:-g, g:-g], Ur[:, g:-g, g:-g]) <= 1e-4
    assert rel_err(Bm[:, g:-g], Br[:, g:-g]) <= 1e-3
    lv.close()
    ctx.close()


SW_STEPS = 1000                     # the slip-weakening workload's max_step


def test_mixed_slip_weakening_rupture_metrics_vs_fp64_oracle(cuda_lib):
    """The slip-weakening workload at full size (512x256, dx = 0.1 km, 1000
    steps, side 2 at offset 11): the mixed form's rupture against the FP64
    oracle's at fault stations 3-15 km either side of the nucleation, with the
    station values interpolated on the device (tmk_stations_*) and by the
    oracle's restatement of the same interpolation."""
    import os
    from tetemoko_gb300 import rupture as R
    from tetemoko_gb300.level import Context, LinElastLevelGodunov
    from tetemoko_gb300.stations import Stations
    sc64 = S.slip_weakening(nx=512, ny=256, dx=0.1)
    scm = S.slip_weakening(nx=512, ny=256, dx=0.1, precision=A.TMK_PREC_MIXED)
    xc = sc64.nx * sc64.dx / 2.0
    fx = [xc + s * d for d in (3.0, 6.0, 9.0, 12.0, 15.0) for s in (-1.0, 1.0)]
    dt = sc64.dt()
    g = A.TMK_NGHOST
    dom = (0, 0, sc64.nx - 1, sc64.ny - 1)
    # FP64 oracle
    U, B = sc64.initial_U(), sc64.initial_B()
    boxes = O.tile_boxes(sc64.nx, sc64.ny, 128)
    nthreads = max(1, len(os.sched_getaffinity(0)))
    ts, Vf = [], []
    t = 0.0
    for _ in range(SW_STEPS):
        assert O.level_step(sc64, U, B, boxes, t, dt, nthreads=nthreads) == 0
        t += dt
        wf, _ = O.station_values(dom, sc64.dx, U, B, fx, [])
        ts.append(t)
        Vf.append(np.asarray(wf))
    ref = {"time": np.array(ts), "fault": np.array(Vf)}
    # mixed form on the device
    ctx = Context(scm)
    lvl = LinElastLevelGodunov(ctx, [dom])
    lvl.set_patch(0, scm.initial_U(), scm.initial_B())
    st = Stations(lvl, fx, [], capacity=SW_STEPS + 8)
    st.attach()
    t = 0.0
    for _ in range(SW_STEPS):
        lvl.step(t, dt)
        t += dt
    rec = st.read()
    Um, _ = lvl.get_patch(0)
    rc, info = lvl.status()
    st.close(); lvl.close(); ctx.close()
    assert rc == 0, info
    thr = sc64.sw.rupture_threshold
    e = R.compare(R.station_metrics(rec, A.TMK_FAULT_SW, thr), R.station_metrics(ref, A.TMK_FAULT_SW, thr))
    vel_err = R.velocity_error(Um, U)
    print(f"slip weakening, mixed vs FP64 oracle, {SW_STEPS} steps: {e}, volume velocity {vel_err:.2e}")
    assert e["stations_ruptured"] == len(fx), "every station must rupture within the run"
    assert e["arrival"] < ARRIVAL_RTOL
    assert e["final_slip"] < SLIP_RTOL
    assert e["peak_slip_rate"] < PEAK_RTOL
    assert vel_err < VEL_RTOL
