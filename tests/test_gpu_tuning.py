"""Level tuning and the autotuner: every work-list shape and fault-kernel
variant computes the same step (the marching kernels and the fault kernel
compute each cell and face by the same arithmetic whatever the cut), the
autotuner leaves the level's state as it found it, and tunings are refused
where they would be unsafe."""
import numpy as np
import pytest

from tetemoko_gb300 import _capi as A, scenarios as S
from tests import amr_helpers as H
from tests.helpers import perturbed_state, rel_err

pytestmark = pytest.mark.gpu
G = A.TMK_NGHOST
BOXES = [(0, 0, 20, 9), (21, 0, 63, 9), (0, 10, 31, 31), (32, 10, 63, 31)]


def _tuning(volume="march", waves=(1, 1), min_run=16, disp=1, seg=32, first=0, fused=0):
    t = A.Tuning()
    t.volume_kernel = A.TMK_VOLUME_MARCH if volume == "march" else A.TMK_VOLUME_TILE
    t.march_waves[0], t.march_waves[1] = waves
    t.min_run, t.fault_displace, t.fault_seg, t.fault_first = min_run, disp, seg, first
    t.plastic_fused = fused
    return t


VARIANTS = [dict(), dict(waves=(2, 1)), dict(waves=(1, 2), min_run=8), dict(min_run=32, disp=0),
            dict(seg=16), dict(waves=(2, 2), min_run=8, disp=2, seg=16), dict(first=1, seg=16, disp=0),
            dict(first=1, seg=32, waves=(2, 1))]


def _run(sc, Ug, Bg, tuning, nsteps=6):
    from tetemoko_gb300.level import Context, LinElastLevelGodunov
    ctx = Context(sc)
    lvl = LinElastLevelGodunov(ctx, BOXES)
    lvl.set_level(Ug, Bg)
    if tuning is not None:
        lvl.set_tuning(tuning)
    dt = sc.dt()
    for k in range(nsteps):
        lvl.step(k * dt, dt)
    U, B = Ug.copy(), Bg.copy()
    lvl.get_level(U, B)
    assert lvl.status()[0] == 0
    lvl.close()
    ctx.close()
    return U, B


@pytest.mark.parametrize("prec", [A.TMK_PREC_FP64, A.TMK_PREC_MIXED], ids=["fp64", "mixed"])
def test_every_marching_tuning_computes_the_same_step(cuda_lib, prec):
    sc = S.rate_state(nx=64, ny=32, dx=0.1, precision=prec)
    rng = np.random.default_rng(41)
    Ug = perturbed_state(sc, rng, amp_v=0.05, amp_s=1.0)
    Bg = sc.initial_B()
    U0, B0 = _run(sc, Ug, Bg, None)
    for v in VARIANTS:
        U, B = _run(sc, Ug, Bg, _tuning(**v))
        np.testing.assert_array_equal(U[:, G:-G, G:-G], U0[:, G:-G, G:-G], err_msg=str(v))
        np.testing.assert_array_equal(B[:, G:-G], B0[:, G:-G], err_msg=str(v))
    # the tile kernel: the same method with another operation order (FP32
    # rounding of a ~1e2 MPa state, amplified by the limiters, in the mixed form)
    U, B = _run(sc, Ug, Bg, _tuning(volume="tile", seg=16))
    tol = 1e-12 if prec == A.TMK_PREC_FP64 else 1e-4
    assert rel_err(U[:, G:-G, G:-G], U0[:, G:-G, G:-G]) <= tol


@pytest.mark.parametrize("prec", [A.TMK_PREC_FP64, A.TMK_PREC_MIXED], ids=["fp64", "mixed"])
def test_plastic_return_fused_or_as_a_pass_computes_the_same_step(cuda_lib, prec):
    """A plastic level: the Drucker-Prager return applied by the in-plane
    marching kernel's stores (antiplane kernel first, fault kernel on a side
    stream) equals the return as a pass after the marching kernels -- bit for
    bit in the FP64 form, to FP32 rounding in the mixed form -- across
    work-list shapes; the state yields somewhere."""
    sc = S.slip_weakening(nx=64, ny=32, dx=0.1, precision=prec, plasticity=True)
    rng = np.random.default_rng(45)
    Ug = perturbed_state(sc, rng, amp_v=0.05, amp_s=1.0)
    for side in (0, 11):                         # shear above the yield stress in a band
        Ug[side + 6, G + 8:G + 14, :] += 60.0
    Bg = sc.initial_B()
    U0, B0 = _run(sc, Ug, Bg, _tuning(fused=0))
    assert U0[9, G:-G, G:-G].max() > 0 and U0[10, G:-G, G:-G].max() > 0, "the state must yield"
    tol = 0.0 if prec == A.TMK_PREC_FP64 else 1e-5
    for v in (dict(fused=1), dict(fused=1, waves=(2, 2), min_run=8, seg=16), dict(fused=0, first=1, disp=0)):
        U, B = _run(sc, Ug, Bg, _tuning(**v))
        assert rel_err(U[:, G:-G, G:-G], U0[:, G:-G, G:-G]) <= tol, v
        assert rel_err(B[:, G:-G], B0[:, G:-G]) <= max(tol, 1e-300), v


def test_plastic_hierarchy_with_the_fused_return_matches_the_pass(cuda_lib):
    """A ratio-4 plastic hierarchy whose levels apply the fused return steps as
    the one with the return as a pass (FP64, bit for bit)."""
    from tetemoko_gb300.amr import AMRHierarchy
    from tetemoko_gb300.level import Context
    from tests.test_gpu_amr import _levels_on_gpu, _read
    sc = S.slip_weakening(nx=64, ny=32, dx=0.1, plasticity=True)
    datas = H.hierarchy(sc, np.random.default_rng(46), nlev=3, ratios=(4, 4))
    ctx = Context(sc)
    res = []
    for fused in (0, 1):
        lvs = _levels_on_gpu(ctx, datas)
        h = AMRHierarchy(lvs, [4, 4])
        for lv in lvs:
            lv.set_tuning(_tuning(fused=fused))
        for _ in range(2):
            h.step(sc.dt())
        res.append([_read(lv, d) for lv, d in zip(lvs, datas)])
        for lv in lvs:
            assert lv.status()[0] == 0
        h.close()
        for lv in lvs:
            lv.close()
    for a, b in zip(*res):
        for p in range(len(a.boxes)):
            np.testing.assert_array_equal(a.U[p][:, G:-G, G:-G], b.U[p][:, G:-G, G:-G])
            if a.B[p] is not None:
                np.testing.assert_array_equal(a.B[p][:, G:-G], b.B[p][:, G:-G])
    ctx.close()


def test_autotune_keeps_the_state_and_picks_a_valid_tuning(cuda_lib):
    from tetemoko_gb300.level import Context, LinElastLevelGodunov
    sc = S.rate_state(nx=64, ny=32, dx=0.1, precision=A.TMK_PREC_MIXED)
    rng = np.random.default_rng(42)
    Ug = perturbed_state(sc, rng, amp_v=0.05, amp_s=1.0)
    Bg = sc.initial_B()
    ctx = Context(sc)
    lvl = LinElastLevelGodunov(ctx, BOXES)
    lvl.set_level(Ug, Bg)
    dt = sc.dt()
    lvl.step(0.0, dt)                      # parity 1: the snapshot must restore it
    Ua, Ba = Ug.copy(), Bg.copy()
    lvl.get_level(Ua, Ba)
    t, ms = lvl.autotune(dt, dt, steps=3)
    assert ms > 0
    d = t.as_dict()
    assert d["volume_kernel"] in ("march", "tile") and d["fault_seg"] in (16, 32)
    assert lvl.tuning().as_dict() == d
    Ub, Bb = Ug.copy(), Bg.copy()
    lvl.get_level(Ub, Bb)
    np.testing.assert_array_equal(Ub, Ua)
    np.testing.assert_array_equal(Bb, Ba)
    assert lvl.status()[0] == 0
    # the tuned level steps as a fresh level with the same tuning
    for k in range(1, 5):
        lvl.step(k * dt, dt)
    Uc, Bc = Ug.copy(), Bg.copy()
    lvl.get_level(Uc, Bc)
    fresh = LinElastLevelGodunov(ctx, BOXES)
    fresh.set_level(Ug, Bg)
    fresh.set_tuning(t)
    for k in range(5):
        fresh.step(k * dt, dt)
    Ud, Bd = Ug.copy(), Bg.copy()
    fresh.get_level(Ud, Bd)
    np.testing.assert_array_equal(Uc[:, G:-G, G:-G], Ud[:, G:-G, G:-G])
    lvl.close()
    fresh.close()
    ctx.close()


def test_tuning_is_refused_where_unsafe(cuda_lib):
    from tetemoko_gb300.level import Context, LinElastLevelGodunov
    sc = S.rate_state(nx=64, ny=32, dx=0.1)
    ctx = Context(sc)
    lvl = LinElastLevelGodunov(ctx, BOXES)
    lvl.set_level(sc.initial_U(), sc.initial_B())
    for bad in (dict(waves=(0, 1)), dict(min_run=2), dict(disp=9), dict(seg=8), dict(first=2), dict(fused=3)):
        with pytest.raises(A.TmkError):
            lvl.set_tuning(_tuning(**bad))
    g = lvl.graph(2, 0.0, sc.dt())
    with pytest.raises(A.TmkError):
        lvl.set_tuning(_tuning(waves=(2, 2)))      # the graph launches the present work lists
    with pytest.raises(A.TmkError):
        lvl.autotune(0.0, sc.dt())
    g.close()
    lvl.set_tuning(_tuning(waves=(2, 2)))
    lvl.close()
    sct = S.rate_state(nx=64, ny=32, dx=0.1)
    sct.scheme.volume_kernel = A.TMK_VOLUME_TILE
    ct = Context(sct)
    lt = LinElastLevelGodunov(ct, BOXES)
    with pytest.raises(A.TmkError):
        lt.set_tuning(_tuning())                   # the scheme does not allow the marching kernels
    lt.close()
    ct.close()
    ctx.close()


def test_tuning_an_attached_level_keeps_the_hierarchy_step(cuda_lib):
    """Retuning levels after they are attached rebuilds their coarse-fine
    capture lists: the subcycled steps are unchanged bit for bit."""
    from tetemoko_gb300.amr import AMRHierarchy
    from tetemoko_gb300.level import Context
    from tests.test_gpu_amr import _levels_on_gpu, _read
    sc = S.rate_state(nx=64, ny=32, dx=0.1)
    datas = H.hierarchy(sc, np.random.default_rng(43), nlev=3)
    ctx = Context(sc)
    res = []
    for tuned in (False, True):
        lvs = _levels_on_gpu(ctx, datas)
        h = AMRHierarchy(lvs, [2, 2])
        if tuned:
            for lv in lvs:
                lv.set_tuning(_tuning(waves=(2, 2), min_run=8, disp=0, seg=16))
        for _ in range(2):
            h.step(sc.dt())
        res.append([_read(lv, d) for lv, d in zip(lvs, datas)])
        h.close()
        for lv in lvs:
            lv.close()
    for a, b in zip(*res):
        for p in range(len(a.boxes)):
            np.testing.assert_array_equal(a.U[p][:, G:-G, G:-G], b.U[p][:, G:-G, G:-G])
    ctx.close()


def test_hierarchy_autotune_keeps_the_state_and_the_steps(cuda_lib):
    """The hierarchy autotuner puts the levels' state and the clock back, and
    the tuned hierarchy steps as the untuned one (bit for bit unless it picked
    the tile kernel for a level)."""
    from tetemoko_gb300.amr import AMRHierarchy
    from tetemoko_gb300.level import Context
    from tests.test_gpu_amr import _levels_on_gpu, _read
    sc = S.rate_state(nx=64, ny=32, dx=0.1)
    datas = H.hierarchy(sc, np.random.default_rng(44), nlev=3)
    ctx = Context(sc)
    la, lb = _levels_on_gpu(ctx, datas), _levels_on_gpu(ctx, datas)
    ha, hb = AMRHierarchy(la, [2, 2]), AMRHierarchy(lb, [2, 2])
    ts, ms = hb.autotune(sc.dt(), ncoarse=1)
    assert ms > 0 and len(ts) == 3
    assert hb.time(0) == 0.0 and hb.time(2) == 0.0
    for lv, d in zip(lb, datas):
        r = _read(lv, d)
        for p in range(len(d.boxes)):
            np.testing.assert_array_equal(r.U[p][:, G:-G, G:-G], d.U[p][:, G:-G, G:-G])
    for _ in range(2):
        ha.step(sc.dt())
        hb.step(sc.dt())
    tile = any(t.volume_kernel == A.TMK_VOLUME_TILE for t in ts)
    for a, b, d in zip(la, lb, datas):
        ra, rb = _read(a, d), _read(b, d)
        for p in range(len(d.boxes)):
            if tile:
                assert rel_err(rb.U[p][:, G:-G, G:-G], ra.U[p][:, G:-G, G:-G]) <= 1e-12
            else:
                np.testing.assert_array_equal(rb.U[p][:, G:-G, G:-G], ra.U[p][:, G:-G, G:-G])
    ha.close(); hb.close()
    for lv in la + lb:
        lv.close()
    ctx.close()
