"""Coarse-fine coupling on the device equals the oracle: ghost fill (space and
time interpolation), average-down, regrid prolongation, and whole subcycled
hierarchy steps with flux registers and reflux (FP64 form, 1e-12 per
operator, 1e-11 after several steps); the mixed form stays within FP32
rounding of the FP64 oracle; refluxing conserves the composite sum."""
import numpy as np
import pytest

import oracle as O
from tetemoko_gb300 import _capi as A, scenarios as S
from tests import amr_helpers as H
from tests.helpers import RTOL_FP64, rel_err

pytestmark = pytest.mark.gpu
G = A.TMK_NGHOST


def _levels_on_gpu(ctx, datas):
    from tetemoko_gb300.level import LinElastLevelGodunov
    out = []
    for d in datas:
        lv = LinElastLevelGodunov(ctx, d.boxes, domain=d.domain, dx=d.dx)
        lv.set_patches(d.U, d.B)
        out.append(lv)
    return out


def _read(lv, like: O.LevelData) -> O.LevelData:
    Us, Bs = lv.get_patches()
    return O.LevelData(like.domain, like.dx, like.boxes, like.nb, Us, Bs)


def _fault_err(a, b) -> float:
    """Per fault component, relative to its largest value with a floor of 1e-3
    (slip rates near zero are differences of O(0.1) face velocities: their
    rounding is absolute; the 100 and 1e10 sentinels must not set the scale)."""
    scale = np.maximum(np.abs(b).max(axis=1), 1e-3)
    return float((np.abs(a - b).max(axis=1) / scale).max())


def _valid_err(a: O.LevelData, b: O.LevelData) -> float:
    e = 0.0
    for p in range(len(a.boxes)):
        e = max(e, rel_err(a.U[p][:, G:-G, G:-G], b.U[p][:, G:-G, G:-G]))
        if b.B[p] is not None:
            e = max(e, _fault_err(a.B[p][:, G:-G], b.B[p][:, G:-G]))
    return e


def _all_err(a: O.LevelData, b: O.LevelData) -> float:
    e = 0.0
    for p in range(len(a.boxes)):
        e = max(e, rel_err(a.U[p], b.U[p]))
        if b.B[p] is not None:
            e = max(e, _fault_err(a.B[p], b.B[p]))
    return e


def _scenario(kind="rs", precision=A.TMK_PREC_FP64):
    if kind == "rs":
        sc = S.rate_state(nx=64, ny=32, dx=0.1, precision=precision)
    elif kind == "sw":
        sc = S.slip_weakening(nx=64, ny=32, dx=0.1, precision=precision)
    elif kind == "sw_ref9":                          # the reference's side-2 layout at component 9
        sc = S.slip_weakening(nx=64, ny=32, dx=0.1, precision=precision, layout=A.TMK_SW_LAYOUT_REFERENCE9)
    elif kind == "sw_plastic":
        sc = S.slip_weakening(nx=64, ny=32, dx=0.1, precision=precision, plasticity=True)
    else:
        raise ValueError(kind)
    return sc


# a ratio's hierarchy layout (the reference decks refine by 4 and 8)
RATIO_LAYOUT = {2: (2, 2), 4: (4, 4), 8: (8,)}
FILL_CASES = [(r, a) for r in (2, 4, 8) for a in (0.0, 0.25, 0.3, 0.5, 0.75, 1.0)]


@pytest.mark.parametrize("r,alpha", FILL_CASES, ids=[f"r{r}_a{a}" for r, a in FILL_CASES])
def test_cf_fill_matches_oracle(cuda_lib, r, alpha):
    from tetemoko_gb300.level import Context
    sc = _scenario()
    rng = np.random.default_rng(21)
    d0, d1 = H.hierarchy(sc, rng, nlev=2, ratios=RATIO_LAYOUT[r])
    for u in d1.U:                                   # ghosts the fill must overwrite (or keep)
        u[:, :G, :] = rng.standard_normal(u[:, :G, :].shape)
        u[:, :, -G:] = rng.standard_normal(u[:, :, -G:].shape)
    ctx = Context(sc)
    C, F = _levels_on_gpu(ctx, [d0, d1])
    F.attach_coarser(C, r)
    C.step(0.0, sc.dt())
    cnew = _read(C, d0)
    F.fill_coarse_fine(alpha)
    got = _read(F, d1)
    ref = d1.copy()
    assert O.cf_fill(r, d0, cnew, alpha, ref) == 0
    assert _all_err(got, ref) <= RTOL_FP64
    F.close(); C.close(); ctx.close()


@pytest.mark.parametrize("r", [2, 4, 8])
def test_cf_time_coefficient_snaps_to_the_coarse_times(cuda_lib, r):
    """LinElastLevelGodunov::step's alpha = (t - tCold) / (tCnew - tCold) is
    snapped to 0 or 1 within 0.04 dt / r (LinElastLevelGodunov.cpp:230-256):
    a fine step that starts just inside the window equals the step taken at
    the coarse time itself; alpha outside [0, 1] after snapping is an error."""
    from tetemoko_gb300.level import Context
    sc = _scenario()
    sc.scheme.fault_law = A.TMK_FAULT_NONE          # rupture times would record the shifted start
    sc.scheme.boundary_type[2] = 0
    d0, d1 = H.hierarchy(sc, np.random.default_rng(27), nlev=2, ratios=RATIO_LAYOUT[r])
    ctx = Context(sc)
    dtc = sc.dt()
    dtf = dtc / r
    outs = []
    eps_t = 0.03 * dtf / r * dtc                 # alpha = 0.03 dt / r: inside the window (0.04 dt / r)
    for t0, edge in ((0.0, 0), (eps_t, 0), (dtc, 1), (dtc - eps_t, 1)):
        C, F = _levels_on_gpu(ctx, [d0, d1])
        F.attach_coarser(C, r)
        C.step(0.0, dtc)
        F.step(t0, dtf, t_coarse_old=0.0, t_coarse_new=dtc)
        outs.append((edge, _read(F, d1)))
        if edge == 1:
            with pytest.raises(A.TmkError):           # alpha > 1 + eps
                F.step(dtc + 0.1 * dtf, dtf, t_coarse_old=0.0, t_coarse_new=dtc)
        F.close(); C.close()
    for e in (0, 1):
        a, b = [o for edge, o in outs if edge == e]
        for p in range(len(a.boxes)):
            np.testing.assert_array_equal(a.U[p], b.U[p])
    # the two ends differ: the test is not vacuous
    assert max(rel_err(outs[0][1].U[p], outs[2][1].U[p]) for p in range(len(d1.boxes))) > 1e-6
    ctx.close()


@pytest.mark.parametrize("r", [2, 4, 8])
def test_average_down_and_prolongation_match_oracle(cuda_lib, r):
    from tetemoko_gb300.level import Context
    sc = _scenario()
    rng = np.random.default_rng(22)
    d0, d1 = H.hierarchy(sc, rng, nlev=2, ratios=RATIO_LAYOUT[r], fine_noise=0.05)
    ctx = Context(sc)
    C, F = _levels_on_gpu(ctx, [d0, d1])
    F.attach_coarser(C, r)
    C.average_down()
    ref = d0.copy()
    assert O.average_down(r, ref, d1) == 0
    assert _valid_err(_read(C, d0), ref) <= RTOL_FP64
    # prolongation of the (averaged) coarse level onto the fine level
    F.interp_from_coarser()
    fref = d1.copy()
    assert O.fine_interp(r, ref, fref) == 0
    assert _valid_err(_read(F, d1), fref) <= RTOL_FP64
    F.close(); C.close(); ctx.close()


REGRID_BOXES = {2: [(48, 0, 79, 15), (48, 16, 79, 27)],
                4: [(128, 0, 191, 31), (128, 32, 159, 55)],
                8: [(256, 0, 383, 47), (384, 0, 415, 23)]}


@pytest.mark.parametrize("r", [2, 4, 8])
def test_regrid_prolongs_then_copies_the_old_level(cuda_lib, r):
    from tetemoko_gb300.amr import regrid_level
    from tetemoko_gb300.level import Context, LinElastLevelGodunov
    sc = _scenario()
    rng = np.random.default_rng(23)
    d0, d1 = H.hierarchy(sc, rng, nlev=2, ratios=RATIO_LAYOUT[r], fine_noise=0.05)
    ctx = Context(sc)
    C, F = _levels_on_gpu(ctx, [d0, d1])
    F.attach_coarser(C, r)
    new_boxes = REGRID_BOXES[r]
    N = LinElastLevelGodunov(ctx, new_boxes, domain=d1.domain, dx=d1.dx)
    regrid_level(N, F, C, r)
    dn = O.LevelData(d1.domain, d1.dx, new_boxes, d1.nb)
    assert O.fine_interp(r, d0, dn) == 0
    for p, nb in enumerate(new_boxes):            # copy of the old fine cells
        for q, ob in enumerate(d1.boxes):
            lo0, hi0, lo1, hi1 = max(nb[0], ob[0]), min(nb[2], ob[2]), max(nb[1], ob[1]), min(nb[3], ob[3])
            if lo0 > hi0 or lo1 > hi1:
                continue
            dst = (slice(None), slice(lo1 - nb[1] + G, hi1 - nb[1] + G + 1), slice(lo0 - nb[0] + G, hi0 - nb[0] + G + 1))
            src = (slice(None), slice(lo1 - ob[1] + G, hi1 - ob[1] + G + 1), slice(lo0 - ob[0] + G, hi0 - ob[0] + G + 1))
            dn.U[p][dst] = d1.U[q][src]
            if dn.B[p] is not None and d1.B[q] is not None:
                dn.B[p][:, lo0 - nb[0] + G:hi0 - nb[0] + G + 1] = d1.B[q][:, lo0 - ob[0] + G:hi0 - ob[0] + G + 1]
    assert _valid_err(_read(N, dn), dn) <= RTOL_FP64
    N.close(); F.close(); C.close(); ctx.close()


CASES = [("rs", (2, 2), 2, 3), ("rs", (2, 2), 3, 2), ("sw", (2, 2), 2, 3), ("sw_plastic", (2, 2), 2, 2),
         ("rs", (4, 4), 2, 2), ("rs", (4, 4), 3, 1), ("sw", (4, 4), 2, 2), ("sw_ref9", (4, 4), 2, 2),
         ("sw_plastic", (4, 4), 2, 2), ("sw_plastic", (4, 4), 3, 1), ("rs", (4, 2), 3, 2),
         ("rs", (8,), 2, 1), ("sw_plastic", (8,), 2, 1)]


@pytest.mark.parametrize("kind,ratios,nlev,nsteps", CASES,
                         ids=[f"{k}_r{'x'.join(map(str, r[:n - 1]))}_{n}lev" for k, r, n, _ in CASES])
def test_amr_hierarchy_matches_oracle(cuda_lib, kind, ratios, nlev, nsteps):
    from tetemoko_gb300.amr import AMRHierarchy
    from tetemoko_gb300.level import Context
    sc = _scenario(kind)
    rng = np.random.default_rng(24)
    datas = H.hierarchy(sc, rng, nlev=nlev, ratios=ratios)
    refs = [d.copy() for d in datas]
    ratios = list(ratios[:nlev - 1])
    assert O.amr_run(sc, refs, ratios, 0.0, sc.dt(), nsteps) == 0
    ctx = Context(sc)
    lvs = _levels_on_gpu(ctx, datas)
    h = AMRHierarchy(lvs, ratios)
    for _ in range(nsteps):
        h.step(sc.dt())
    assert abs(h.time(nlev - 1) - nsteps * sc.dt()) < 1e-12
    for lv, d, r in zip(lvs, datas, refs):
        rc, info = lv.status()
        assert rc == 0, info
        assert _valid_err(_read(lv, d), r) <= 1e-11
    sub = np.cumprod([1] + ratios)
    assert h.cell_updates() == sum(
        sum((b[2] - b[0] + 1) * (b[3] - b[1] + 1) for b in d.boxes) * int(sub[l]) for l, d in enumerate(datas))
    h.close()
    for lv in lvs:
        lv.close()
    ctx.close()


MIXED_CASES = [("rs", (2,)), ("rs", (4,)), ("sw_plastic", (4, 4))]


@pytest.mark.parametrize("kind,ratios", MIXED_CASES, ids=[f"{k}_r{'x'.join(map(str, r))}" for k, r in MIXED_CASES])
def test_amr_mixed_form_within_fp32_rounding(cuda_lib, kind, ratios):
    from tetemoko_gb300.amr import AMRHierarchy
    from tetemoko_gb300.level import Context
    sc = _scenario(kind)
    rng = np.random.default_rng(25)
    datas = H.hierarchy(sc, rng, nlev=len(ratios) + 1, ratios=RATIO_LAYOUT[ratios[0]])
    refs = [d.copy() for d in datas]
    assert O.amr_run(sc, refs, list(ratios), 0.0, sc.dt(), 3) == 0
    sc.scheme.precision = A.TMK_PREC_MIXED
    ctx = Context(sc)
    lvs = _levels_on_gpu(ctx, datas)
    h = AMRHierarchy(lvs, list(ratios))
    for _ in range(3):
        h.step(sc.dt())
    for lv, d, r in zip(lvs, datas, refs):
        assert lv.status()[0] == 0
        got = _read(lv, d)
        for p in range(len(d.boxes)):
            assert rel_err(got.U[p][:, G:-G, G:-G], r.U[p][:, G:-G, G:-G]) <= 1e-4
            if r.B[p] is not None:
                assert rel_err(got.B[p][:, G:-G], r.B[p][:, G:-G]) <= 1e-3
    h.close()
    for lv in lvs:
        lv.close()
    ctx.close()


@pytest.mark.parametrize("r", [2, 4])
def test_amr_refluxing_conserves_the_composite_sum_on_device(cuda_lib, r):
    from tetemoko_gb300.amr import AMRHierarchy
    from tetemoko_gb300.level import Context
    from tests.test_oracle_amr import _bump_level, _no_fault_bump
    sc = _no_fault_bump()
    fboxes = [(16 * r, 8 * r, 32 * r - 1, 16 * r - 1), (16 * r, 16 * r, 32 * r - 1, 24 * r - 1)]
    C0 = _bump_level(sc, (0, 0, 47, 31), 0.2, O.tile_boxes(48, 32, 16), 3.2, 3.2, 0.6)
    F0 = _bump_level(sc, (0, 0, 48 * r - 1, 32 * r - 1), 0.2 / r, fboxes, 3.2, 3.2, 0.6)
    ctx = Context(sc)
    C, F = _levels_on_gpu(ctx, [C0, F0])
    h = AMRHierarchy([C, F], [r])
    t0 = H.composite_sum([C0, F0], [r])
    for _ in range(2):
        h.step(sc.dt())
    t1 = H.composite_sum([_read(C, C0), _read(F, F0)], [r])
    assert (np.abs(t1 - t0) / np.maximum(np.abs(t0), 1.0)).max() < 1e-14
    h.close(); F.close(); C.close(); ctx.close()


def test_attach_rejects_bad_layouts(cuda_lib):
    from tetemoko_gb300.level import Context, LinElastLevelGodunov
    sc = _scenario()
    ctx = Context(sc)
    C = LinElastLevelGodunov(ctx, H.L0_BOXES)
    F = LinElastLevelGodunov(ctx, [(41, 0, 71, 15)], domain=(0, 0, 127, 63), dx=0.05)     # not aligned to 2
    with pytest.raises(A.TmkError):
        F.attach_coarser(C, 2)
    F2 = LinElastLevelGodunov(ctx, [(40, 0, 71, 15)], domain=(0, 0, 127, 63), dx=0.05)
    F2.attach_coarser(C, 2)
    with pytest.raises(A.TmkError):          # a level with a coarser level needs the coarse times
        F2.step(0.0, sc.dt() / 2)
    F2.close(); F.close(); C.close(); ctx.close()


def test_amr_per_face_friction(cuda_lib):
    """Per-face friction on every level of a subcycled hierarchy (mixed form):
    values equal to the scenario's constants give the constant run bit for bit;
    a +-10% field, refined piecewise constant onto the finer level, changes it."""
    from tetemoko_gb300.amr import AMRHierarchy
    from tetemoko_gb300.level import Context
    sc = _scenario("rs", A.TMK_PREC_MIXED)
    datas = H.hierarchy(sc, np.random.default_rng(26), nlev=2)
    ctx = Context(sc)
    out = []
    for mode in ("none", "const", "field"):
        lvs = _levels_on_gpu(ctx, datas)
        for l, lv in enumerate(lvs):
            if mode == "none":
                continue
            F = S.friction_field(sc, refine=2 ** l)
            if mode == "const":
                F = np.tile(np.array([sc.rs.a, sc.rs.b, sc.rs.L])[:, None], (1, F.shape[1]))
            lv.set_level_friction(F)
        h = AMRHierarchy(lvs, [2])
        for _ in range(3):
            h.step(sc.dt())
        out.append([_read(lv, d) for lv, d in zip(lvs, datas)])
        for lv in lvs:
            assert lv.status()[0] == 0
        h.close()
        for lv in lvs:
            lv.close()
    for a, b, c in zip(*out):
        for p in range(len(a.boxes)):
            np.testing.assert_array_equal(a.U[p], b.U[p])
            if a.B[p] is not None:
                np.testing.assert_array_equal(a.B[p], b.B[p])
    fine_a, fine_c = out[0][1], out[2][1]
    diffs = [rel_err(fine_c.B[p][10:11, G:-G], fine_a.B[p][10:11, G:-G])
             for p in range(len(fine_a.boxes)) if fine_a.B[p] is not None]
    assert diffs and max(diffs) > 1e-9
    ctx.close()
