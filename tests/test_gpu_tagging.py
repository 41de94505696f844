"""Refinement tagging on the device == the oracle's restatement of
AMRLevelLinElast::tagCells / tagCellsInit, bit for bit in the FP64 form
(single levels, a fine level filled from its coarser level, the plastic
strain and coarsening tests, the tag buffer)."""
import numpy as np
import pytest

import oracle as O
from tetemoko_gb300 import _capi as A, scenarios as S
from tests import amr_helpers as H
from tests.helpers import perturbed_state

pytestmark = pytest.mark.gpu
G = A.TMK_NGHOST
BOXES = [(0, 0, 20, 9), (21, 0, 63, 9), (0, 10, 31, 31), (32, 10, 63, 31)]


def _device_level(sc, Ug, Bg):
    from tetemoko_gb300.level import Context, LinElastLevelGodunov
    ctx = Context(sc)
    lvl = LinElastLevelGodunov(ctx, BOXES)
    lvl.set_level(Ug, Bg)
    return ctx, lvl


@pytest.mark.parametrize("kind", ["rs", "sw"])
@pytest.mark.parametrize("initial", [False, True], ids=["tagCells", "tagCellsInit"])
def test_level_tags_match_oracle(cuda_lib, kind, initial):
    sc = S.rate_state(nx=64, ny=32, dx=0.1) if kind == "rs" else S.slip_weakening(nx=64, ny=32, dx=0.1)
    rng = np.random.default_rng(51)
    Ug = perturbed_state(sc, rng, amp_v=0.05, amp_s=1.0)
    Ug[10, G + 20, G + 40] = 3e-5                 # plastic strain, side 1
    Bg = sc.initial_B()
    ctx, lvl = _device_level(sc, Ug, Bg)
    d = H.level_from_global((0, 0, sc.nx - 1, sc.ny - 1), sc.dx, BOXES, sc.nbdry, Ug, Bg)
    for tp in (A.tag_params(initial=initial, refine_thresh=0.04, tag_buffer=2),
               A.tag_params(initial=initial, refine_thresh=0.02, tag_buffer=0, x_coarsen=(1.0, 4.0),
                            y_coarsen=(-1.0, 1.5), slope_coarsen=2.0, width_coarsen=0.5),
               A.tag_params(initial=initial, level=2, refine_thresh=0.03, tag_buffer=3, coarsen2_max_level=1,
                            x_coarsen2=(0.5, 5.0), y_coarsen2=(-1.0, 2.0))):
        want = O.tag_cells(sc, tp, d.copy())
        got = lvl.tag_cells(tp)
        assert 0 < want.sum() < want.size
        np.testing.assert_array_equal(got, want)
    lvl.close()
    ctx.close()


def test_fine_level_tags_after_the_coarse_fine_fill(cuda_lib):
    """A fine level's tags need its coarse-fine ghost cells (filled from the
    coarser level's state) and its exchanged ghost cells."""
    from tetemoko_gb300.level import Context, LinElastLevelGodunov
    from tests.test_gpu_amr import _levels_on_gpu
    sc = S.rate_state(nx=64, ny=32, dx=0.1)
    datas = H.hierarchy(sc, np.random.default_rng(52), nlev=2, fine_noise=0.05)
    ctx = Context(sc)
    lvs = _levels_on_gpu(ctx, datas)
    lvs[1].attach_coarser(lvs[0], 2)
    tp = A.tag_params(level=1, refine_thresh=0.05, tag_buffer=2)
    want = O.tag_cells(sc, tp, datas[1].copy(), coarse=datas[0], r=2)
    got = lvs[1].tag_cells(tp)
    assert 0 < want.sum() < want.size
    np.testing.assert_array_equal(got, want)
    # the tags on a device buffer
    import torch
    dm = torch.zeros(want.shape, dtype=torch.uint8, device="cuda")
    lvs[1].tag_cells(tp, mask=dm)
    np.testing.assert_array_equal(dm.cpu().numpy(), want)
    for lv in lvs:
        lv.close()
    ctx.close()


def test_mixed_form_tags_agree_away_from_the_threshold(cuda_lib):
    sc = S.rate_state(nx=64, ny=32, dx=0.1, precision=A.TMK_PREC_MIXED)
    rng = np.random.default_rng(53)
    Ug = perturbed_state(sc, rng, amp_v=0.05, amp_s=1.0)
    Bg = sc.initial_B()
    ctx, lvl = _device_level(sc, Ug, Bg)
    d = H.level_from_global((0, 0, sc.nx - 1, sc.ny - 1), sc.dx, BOXES, sc.nbdry, Ug, Bg)
    tp = A.tag_params(refine_thresh=0.04, tag_buffer=0)
    want = O.tag_cells(sc, tp, d)
    got = lvl.tag_cells(tp)
    assert (got != want).mean() <= 0.01
    lvl.close()
    ctx.close()


@pytest.mark.parametrize("kind", ["rs", "sw"])
def test_slip_rate_tags_match_oracle(cuda_lib, kind):
    """The slip-rate tag of the fault row (an extension the refinement of a
    rupture front uses): bit for bit with the oracle, alone and with the
    gradient tags, across the fault row split between patches."""
    sc = S.rate_state(nx=64, ny=32, dx=0.1) if kind == "rs" else S.slip_weakening(nx=64, ny=32, dx=0.1)
    rng = np.random.default_rng(54)
    Ug = perturbed_state(sc, rng, amp_v=0.05, amp_s=1.0)
    Bg = sc.initial_B()
    vc = 2 if kind == "rs" else 4
    x = (np.arange(-G, sc.nx + G) + 0.5) * sc.dx
    Bg[vc] = np.where((x > 1.5) & (x < 2.6), 2e-3, 1e-9) + np.where((x > 4.0) & (x < 4.3), 5e-4, 0.0)
    ctx, lvl = _device_level(sc, Ug, Bg)
    d = H.level_from_global((0, 0, sc.nx - 1, sc.ny - 1), sc.dx, BOXES, sc.nbdry, Ug, Bg)
    for tp in (A.tag_params(refine_thresh=1e10, tag_buffer=0, slip_rate_thresh=1e-3),
               A.tag_params(refine_thresh=1e10, tag_buffer=2, slip_rate_thresh=4e-4),
               A.tag_params(refine_thresh=0.04, tag_buffer=1, slip_rate_thresh=1e-3)):
        want = O.tag_cells(sc, tp, d.copy())
        got = lvl.tag_cells(tp)
        assert want.sum() > 0
        np.testing.assert_array_equal(got, want)
    lvl.close()
    ctx.close()
