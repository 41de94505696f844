"""Known-answer tests of the oracle's AMR operators (CPU).

Properties the reference's coarse-fine operators have by construction:
piecewise-linear prolongation and ghost filling reproduce linear data (the
limiter is inactive on it), averaging undoes prolongation, the fill uses the
coarse states at alpha = 0 / 1 exactly and touches only ghosts no fine patch
covers, and refluxing makes the composite sum of U conserved.
"""
import numpy as np
import pytest

import oracle as O
from tetemoko_gb300 import _capi as A, scenarios as S
from tests import amr_helpers as H

G = A.TMK_NGHOST
CDOM = (0, 0, 31, 15)
CBOXES = [(0, 0, 15, 15), (16, 0, 31, 15)]
FDOM = (0, 0, 63, 31)
FBOXES = [(16, 0, 31, 11), (32, 0, 47, 11)]


def _lin(x, y, c):
    return 1.0 + 0.3 * c + 0.01 * (c + 1) * x - 0.02 * y


def _linear_level(domain, dx, boxes, nb, scale=1.0, shift=0.0):
    L = O.LevelData(domain, dx, boxes, nb)
    for p, b in enumerate(boxes):
        yy, xx = np.mgrid[b[1] - G:b[3] + G + 1, b[0] - G:b[2] + G + 1]
        for c in range(22):
            L.U[p][c] = _lin((xx + 0.5) * scale, (yy + 0.5) * scale, c) + shift
        if L.B[p] is not None:
            xs = np.arange(b[0] - G, b[2] + G + 1)
            for c in range(nb):
                L.B[p][c] = 2.0 + 0.05 * c * (xs + 0.5) * scale + shift
    return L


def test_fine_interp_reproduces_linear_data():
    C = _linear_level(CDOM, 0.2, CBOXES, 11)
    F = O.LevelData(FDOM, 0.1, FBOXES, 11)
    assert O.fine_interp(2, C, F) == 0
    E = _linear_level(FDOM, 0.1, FBOXES, 11, scale=0.5)
    for p in range(len(FBOXES)):
        np.testing.assert_allclose(F.U[p][:, G:-G, G:-G], E.U[p][:, G:-G, G:-G], rtol=0, atol=1e-13)
        np.testing.assert_allclose(F.B[p][:, G:-G], E.B[p][:, G:-G], rtol=0, atol=1e-13)


@pytest.mark.parametrize("r", [2, 4])
def test_average_down_undoes_fine_interp(r):
    rng = np.random.default_rng(11)
    C = O.LevelData(CDOM, 0.2, CBOXES, 11)
    for u in C.U:
        u[:] = rng.standard_normal(u.shape)
    for b in C.B:
        b[:] = rng.standard_normal(b.shape)
    fdom = H.refine_domain(CDOM, r)
    fboxes = [(8 * r, 0, 16 * r - 1, 6 * r - 1), (16 * r, 0, 24 * r - 1, 6 * r - 1)]
    F = O.LevelData(fdom, 0.2 / r, fboxes, 11)
    assert O.fine_interp(r, C, F) == 0
    C2 = C.copy()
    for u in C2.U:
        u[:] = 0.0
    for b in C2.B:
        b[:] = 0.0
    assert O.average_down(r, C2, F) == 0
    for p, cb in enumerate(CBOXES):
        for fb in fboxes:
            lo0, hi0 = max(cb[0], fb[0] // r), min(cb[2], fb[2] // r)
            lo1, hi1 = max(cb[1], fb[1] // r), min(cb[3], fb[3] // r)
            if lo0 > hi0 or lo1 > hi1:
                continue
            sl = (slice(None), slice(lo1 - cb[1] + G, hi1 - cb[1] + G + 1), slice(lo0 - cb[0] + G, hi0 - cb[0] + G + 1))
            np.testing.assert_allclose(C2.U[p][sl], C.U[p][sl], rtol=0, atol=1e-14)
            bs = (slice(None), slice(lo0 - cb[0] + G, hi0 - cb[0] + G + 1))
            np.testing.assert_allclose(C2.B[p][bs], C.B[p][bs], rtol=0, atol=1e-14)


def test_cf_fill_interpolates_in_time_and_space():
    Cold = _linear_level(CDOM, 0.2, CBOXES, 11)
    Cnew = _linear_level(CDOM, 0.2, CBOXES, 11, shift=1.0)
    F0 = O.LevelData(FDOM, 0.1, FBOXES, 11)
    for u in F0.U:
        u[:] = -7.0
    for b in F0.B:
        b[:] = -7.0
    for alpha in (0.0, 0.25, 1.0):
        F = F0.copy()
        assert O.cf_fill(2, Cold, Cnew, alpha, F) == 0
        E = _linear_level(FDOM, 0.1, FBOXES, 11, scale=0.5, shift=alpha)
        for p, b in enumerate(FBOXES):
            changed = F.U[p] != -7.0
            # valid cells and ghosts covered by the other fine patch are untouched
            assert not changed[:, G:-G, G:-G].any()
            yy, xx = np.mgrid[b[1] - G:b[3] + G + 1, b[0] - G:b[2] + G + 1]
            other = np.zeros(xx.shape, bool)
            for q, ob in enumerate(FBOXES):
                if q != p:
                    other |= (xx >= ob[0]) & (xx <= ob[2]) & (yy >= ob[1]) & (yy <= ob[3])
            outside = (xx < FDOM[0]) | (xx > FDOM[2]) | (yy < FDOM[1]) | (yy > FDOM[3])
            expect = ~(other | outside)
            expect[G:-G, G:-G] = False
            assert (changed[0] == expect).all()
            np.testing.assert_allclose(F.U[p][:, expect], E.U[p][:, expect], rtol=0, atol=1e-13)
            bchanged = F.B[p][0] != -7.0
            np.testing.assert_allclose(F.B[p][:, bchanged], E.B[p][:, bchanged], rtol=0, atol=1e-13)
            assert bchanged.sum() > 0


def test_register_entries_count_coarse_fine_faces():
    C = O.LevelData(CDOM, 0.2, CBOXES, 0)
    F = O.LevelData(FDOM, 0.1, FBOXES, 0)
    # fine region = coarse cells x 8..23, y 0..5: 6 faces left, 6 right, 16 above (the fault row is the domain edge)
    assert O.register_entries(2, C, F) == 28


def test_fill_requires_proper_nesting():
    C = O.LevelData(CDOM, 0.2, [(0, 0, 15, 15)], 11)          # the coarse level misses x >= 16
    F = O.LevelData(FDOM, 0.1, [(16, 0, 31, 11)], 11)
    assert O.cf_fill(2, C, C, 1.0, F) == 3


def _no_fault_bump(sc_dx=0.2):
    sc = S.rate_state(nx=48, ny=32, dx=sc_dx)
    sc.scheme.fault_law = A.TMK_FAULT_NONE
    for k in range(6):
        sc.scheme.boundary_type[k] = 0
    return sc


def _bump_level(sc, domain, dx, boxes, x0, y0, R):
    L = O.LevelData(domain, dx, boxes, 0)
    for p, b in enumerate(boxes):
        yy, xx = np.mgrid[b[1] - G:b[3] + G + 1, b[0] - G:b[2] + G + 1]
        rr = np.hypot((xx + 0.5) * dx - x0, (yy + 0.5) * dx - y0)
        f = np.where(rr < R, np.cos(0.5 * np.pi * rr / R) ** 2, 0.0)
        L.U[p][:] = sc.background()[:, None, None]
        for c, a in ((0, 0.5), (1, -0.3), (2, 0.2), (6, 2.0), (11, 0.4), (15, 1.5), (19, 0.7)):
            L.U[p][c] += a * f
    return L


@pytest.mark.parametrize("r", [2, 4, 8])
def test_amr_refluxing_conserves_the_composite_sum(r):
    """No fault, absorbing edges, a compact pulse straddling the coarse-fine
    boundary: the waves stay inside the domain, so the composite sum of every
    conserved component is constant up to rounding (ratios 2, 4 and 8: the r
    fine faces per coarse face and r substeps per coarse step of the register)."""
    sc = _no_fault_bump()
    fdom = (0, 0, 48 * r - 1, 32 * r - 1)
    fboxes = [(16 * r, 8 * r, 32 * r - 1, 16 * r - 1), (16 * r, 16 * r, 32 * r - 1, 24 * r - 1)]
    C = _bump_level(sc, (0, 0, 47, 31), 0.2, O.tile_boxes(48, 32, 16), 3.2, 3.2, 0.6)
    F = _bump_level(sc, fdom, 0.2 / r, fboxes, 3.2, 3.2, 0.6)
    t0 = H.composite_sum([C, F], [r])
    assert O.amr_run(sc, [C, F], [r], 0.0, sc.dt(), 2) == 0
    t1 = H.composite_sum([C, F], [r])
    scale = np.maximum(np.abs(t0), 1.0)
    assert (np.abs(t1 - t0) / scale).max() < 1e-14
    # the pulse moved: the test is not vacuous
    assert np.abs(F.U[0][0] - _bump_level(sc, fdom, 0.2 / r, fboxes[:1], 3.2, 3.2, 0.6).U[0][0]).max() > 1e-3


def test_amr_with_fine_level_covering_the_domain_equals_a_fine_single_level():
    """A finer level that covers the whole domain never reads the coarse level:
    its two substeps equal two single-level steps at the fine resolution."""
    sc = S.rate_state(nx=64, ny=32, dx=0.05)
    rng = np.random.default_rng(3)
    from tests.helpers import perturbed_state
    Ug = perturbed_state(sc, rng, amp_v=0.05, amp_s=1.0)
    Bg = sc.initial_B()
    fboxes = O.tile_boxes(64, 32, 16)
    F = H.level_from_global((0, 0, 63, 31), 0.05, fboxes, sc.nbdry, Ug, Bg)
    C = O.LevelData((0, 0, 31, 15), 0.1, O.tile_boxes(32, 16, 16), sc.nbdry)
    assert O.average_down(2, C, F) == 0
    dt_f = sc.dt()
    assert O.amr_run(sc, [C, F], [2], 0.0, 2 * dt_f, 1) == 0
    Ur, Br = Ug.copy(), Bg.copy()
    for k in range(2):
        assert O.level_step(sc, Ur, Br, fboxes, k * dt_f, dt_f) == 0
    R = H.level_from_global((0, 0, 63, 31), 0.05, fboxes, sc.nbdry, Ur, Br)
    for p in range(len(fboxes)):
        np.testing.assert_array_equal(F.U[p][:, G:-G, G:-G], R.U[p][:, G:-G, G:-G])
        if R.B[p] is not None:
            np.testing.assert_array_equal(F.B[p][:, G:-G], R.B[p][:, G:-G])


def test_amr_three_levels_runs_and_stays_finite():
    sc = S.rate_state(nx=64, ny=32, dx=0.1)
    levels = H.hierarchy(sc, np.random.default_rng(4), nlev=3)
    assert O.amr_run(sc, levels, [2, 2], 0.0, sc.dt(), 2) == 0
    for lv in levels:
        for u in lv.U:
            assert np.isfinite(u[:, G:-G, G:-G]).all()


# ------------------------------------------------------------------ tagging
def _level_of(sc, boxes, U_fn=None):
    d = O.LevelData((0, 0, sc.nx - 1, sc.ny - 1), sc.dx, boxes, sc.nbdry)
    for p, b in enumerate(d.boxes):
        d.U[p][:] = sc.initial_U(lo=b[:2], hi=b[2:])
        if d.B[p] is not None:
            d.B[p][:] = sc.initial_B(xlo=b[0], xhi=b[2])
    return d


def test_initial_tags_are_the_nucleation_cells_grown():
    """tagCellsInit: RS marks [floor(x0/dx), ceil(x0/dx)] on row 0; SW marks each
    nucleation patch's range; both grown by the tag buffer and clipped to the domain."""
    sc = S.rate_state(nx=64, ny=32, dx=0.1)
    sc.rs.x0 = 3.25                          # between cells 32 and 33
    m = O.tag_cells(sc, A.tag_params(initial=True, tag_buffer=1), _level_of(sc, [(0, 0, 63, 31)]))
    want = np.zeros_like(m)
    want[0:2, 31:35] = 1                     # cells 32..33 on row 0, grown by 1 (row -1 clipped)
    assert np.array_equal(m, want)
    sw = S.slip_weakening(nx=64, ny=32, dx=0.1)
    m = O.tag_cells(sw, A.tag_params(initial=True, tag_buffer=0), _level_of(sw, [(0, 0, 31, 31), (32, 0, 63, 31)]))
    c, xc, xw = sw.sw.fric_box_center[0], sw.sw.xc[0], sw.sw.xw[0]
    lo, hi = int(np.floor((c + xc - xw) / sw.dx)), int(np.ceil((c + xc + xw) / sw.dx))
    assert set(np.nonzero(m[0])[0]) == set(range(lo, hi + 1)) and m[1:].sum() == 0


def test_gradient_tags_follow_getfullgradf():
    """A velocity ramp of slope s cells^-1 gives undivided differences of s in
    the interior (central) and on the domain edges (one-sided): every cell
    tags when s >= thresh, none when s < thresh; the plastic strain and the
    coarsening window tag as their tests say."""
    sc = S.rate_state(nx=48, ny=24, dx=0.1)
    sc.rs.x0 = -100.0                        # no nucleation marks inside the domain
    boxes = [(0, 0, 23, 23), (24, 0, 47, 23)]
    for s, expect in ((0.02, 1), (0.005, 0)):
        d = _level_of(sc, boxes)
        for p, b in enumerate(d.boxes):
            i = np.arange(b[0] - 4, b[2] + 5)
            d.U[p][1] = s * i[None, :]           # vy ramp along x
        m = O.tag_cells(sc, A.tag_params(refine_thresh=0.01, tag_buffer=0), d)
        assert (m == expect).all()
    d = _level_of(sc, boxes)
    d.U[1][21, 4 + 5, 4 + 6] = 2e-5              # side-2 plastic strain at cell (30, 5)
    m = O.tag_cells(sc, A.tag_params(refine_thresh=0.01, tag_buffer=0), d)
    assert m.sum() == 1 and m[5, 30] == 1
    # coarsening: the threshold grows by slope*r/width outside [x0, x1]
    d = _level_of(sc, boxes)
    for p, b in enumerate(d.boxes):
        i = np.arange(b[0] - 4, b[2] + 5)
        d.U[p][0] = 0.02 * i[None, :]
    tp = A.tag_params(refine_thresh=0.01, tag_buffer=0, x_coarsen=(0.0, 2.0), slope_coarsen=1.0, width_coarsen=0.1)
    m = O.tag_cells(sc, tp, d)
    x = np.arange(48) * sc.dx
    thr = 0.01 * (1 + np.maximum(0.0, x - 2.0) * 1.0 / 0.1)
    assert np.array_equal(m[0], (0.02 >= thr).astype(np.uint8))


def test_slip_rate_tags_by_hand():
    """The slip-rate tag (an extension): exactly the fault-row cells whose face
    slips at least the threshold, grown by the tag buffer; off when <= 0."""
    G = A.TMK_NGHOST
    boxes = [(0, 0, 20, 9), (21, 0, 63, 9), (0, 10, 31, 31), (32, 10, 63, 31)]
    for sc, vc in ((S.rate_state(nx=64, ny=32, dx=0.1), 2), (S.slip_weakening(nx=64, ny=32, dx=0.1), 4)):
        Ug, Bg = sc.initial_U(), sc.initial_B()
        x = (np.arange(-G, sc.nx + G) + 0.5) * sc.dx
        Bg[vc] = np.where((x > 1.5) & (x < 2.6), 2e-3, 1e-9)
        d = H.level_from_global((0, 0, 63, 31), sc.dx, boxes, sc.nbdry, Ug, Bg)
        m = O.tag_cells(sc, A.tag_params(refine_thresh=1e10, tag_buffer=0, slip_rate_thresh=1e-3), d.copy())
        want = np.zeros_like(m)
        want[0, 15:26] = 1                                  # cell centres 1.55 .. 2.55 km
        np.testing.assert_array_equal(m, want)
        m = O.tag_cells(sc, A.tag_params(refine_thresh=1e10, tag_buffer=2, slip_rate_thresh=1e-3), d.copy())
        want = np.zeros_like(m)
        want[0:3, 13:28] = 1
        np.testing.assert_array_equal(m, want)
        m = O.tag_cells(sc, A.tag_params(refine_thresh=1e10, tag_buffer=2, slip_rate_thresh=0.0), d.copy())
        assert m.sum() == 0
