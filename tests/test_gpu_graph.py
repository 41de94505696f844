"""Recorded CUDA graphs of level steps and of subcycled AMR steps replay the
same computation as stepping call by call (the fault kernels' start times are
shifted to each replay's start)."""
import numpy as np
import pytest

import oracle as O
from tetemoko_gb300 import _capi as A, scenarios as S
from tests import amr_helpers as H
from tests.helpers import perturbed_state, rel_err

pytestmark = pytest.mark.gpu
G = A.TMK_NGHOST


def _level(sc, Ug, Bg, boxes):
    from tetemoko_gb300.level import Context, LinElastLevelGodunov
    ctx = Context(sc)
    lvl = LinElastLevelGodunov(ctx, boxes)
    lvl.set_level(Ug, Bg)
    return ctx, lvl


@pytest.mark.parametrize("prec", [A.TMK_PREC_FP64, A.TMK_PREC_MIXED], ids=["fp64", "mixed"])
def test_level_graph_replays_the_steps(cuda_lib, prec):
    sc = S.rate_state(nx=64, ny=32, dx=0.1, precision=prec)
    rng = np.random.default_rng(31)
    Ug = perturbed_state(sc, rng, amp_v=0.05, amp_s=1.0)
    Bg = sc.initial_B()
    dt = sc.dt()
    ca, la = _level(sc, Ug, Bg, H.L0_BOXES)
    cb, lb = _level(sc, Ug, Bg, H.L0_BOXES)
    for k in range(6):
        la.step(k * dt, dt)
    g = lb.graph(2, 0.0, dt)
    for r in range(3):
        g.launch(2 * r * dt)
    Ua, Ba = Ug.copy(), Bg.copy()
    Ub, Bb = Ug.copy(), Bg.copy()
    la.get_level(Ua, Ba)
    lb.get_level(Ub, Bb)
    vs = (slice(None), slice(G, -G), slice(G, -G))
    np.testing.assert_array_equal(Ub[vs], Ua[vs])
    assert rel_err(Bb[:, G:-G], Ba[:, G:-G]) <= 1e-14     # rupture times: t0 + k dt summed differently
    for lv in (la, lb):
        rc, info = lv.status()
        assert rc == 0, info
    g.close()
    la.close(); lb.close(); ca.close(); cb.close()


def test_level_graph_needs_an_even_step_count(cuda_lib):
    sc = S.rate_state(nx=64, ny=32, dx=0.1)
    ctx, lvl = _level(sc, sc.initial_U(), sc.initial_B(), [(0, 0, 63, 31)])
    with pytest.raises(A.TmkError):
        lvl.graph(3, 0.0, sc.dt())
    lvl.close(); ctx.close()


@pytest.mark.parametrize("kind,ratios", [("rs", (2, 2)), ("sw_plastic", (2, 2)), ("rs", (4, 4)),
                                         ("sw_plastic", (4, 2))])
def test_amr_graph_replays_subcycled_steps(cuda_lib, kind, ratios):
    from tetemoko_gb300.amr import AMRHierarchy
    from tetemoko_gb300.level import Context
    from tests.test_gpu_amr import _fault_err, _levels_on_gpu, _read
    sc = S.rate_state(nx=64, ny=32, dx=0.1) if kind == "rs" else \
        S.slip_weakening(nx=64, ny=32, dx=0.1, plasticity=True)
    datas = H.hierarchy(sc, np.random.default_rng(32), nlev=3, ratios=ratios)
    ctx = Context(sc)
    la = _levels_on_gpu(ctx, datas)
    lb = _levels_on_gpu(ctx, datas)
    ha = AMRHierarchy(la, list(ratios))
    hb = AMRHierarchy(lb, list(ratios))
    for _ in range(4):
        ha.step(sc.dt())
    g = hb.graph(2, sc.dt())
    g.launch(0.0)
    g.launch(2 * sc.dt())
    assert abs(hb.time(2) - ha.time(2)) < 1e-12
    # the coarse-fine time coefficients of the replayed steps were computed from
    # the recording's clock, the call-by-call run's from its own: equal to rounding
    for a, b, d in zip(la, lb, datas):
        ra, rb = _read(a, d), _read(b, d)
        for p in range(len(d.boxes)):
            assert rel_err(rb.U[p][:, G:-G, G:-G], ra.U[p][:, G:-G, G:-G]) <= 1e-12
            if ra.B[p] is not None:
                assert _fault_err(rb.B[p][:, G:-G], ra.B[p][:, G:-G]) <= 1e-11
    g.close()
    ha.close(); hb.close()
    for lv in la + lb:
        lv.close()
    ctx.close()
