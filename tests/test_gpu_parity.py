"""FP64 GPU path == CPU oracle, through the C ABI (the parity tests proper).

Tolerance: 1e-12 relative per component (tests/helpers.py RTOL_FP64); the
FP64 kernels are built without FMA contraction and follow the reference's
operation order, so the remaining differences are last-ulp differences of
the transcendental functions in the friction solve.
"""
import numpy as np
import pytest

import oracle as O
from tetemoko_gb300 import _capi as A, scenarios as S
from tests.helpers import RTOL_FP64, perturbed_state, rel_err

pytestmark = pytest.mark.gpu


def _scenarios():
    out = []
    sc = S.rate_state(nx=64, ny=32, dx=0.1, state_law=A.TMK_RS_SLIP_LAW)
    sc.rs.L = 0.5
    out.append(("rs_slip", sc))
    out.append(("rs_aging", S.rate_state(nx=64, ny=32, dx=0.1)))
    out.append(("sw_ref9", S.slip_weakening(nx=64, ny=32, dx=0.1, layout=A.TMK_SW_LAYOUT_REFERENCE9)))
    out.append(("sw_off11", S.slip_weakening(nx=64, ny=32, dx=0.1, layout=A.TMK_SW_LAYOUT_OFFSET11)))
    sc = S.slip_weakening(nx=64, ny=32, dx=0.1)
    sc.scheme.use_prim_limiting, sc.scheme.use_char_limiting = 0, 1
    out.append(("sw_charlim", sc))
    sc = S.rate_state(nx=64, ny=32, dx=0.1)
    for k, v in enumerate((1, 1, 2, 1, 0, 0)):
        sc.scheme.boundary_type[k] = v
    out.append(("rs_free_edges", sc))
    sc = S.rate_state(nx=64, ny=32, dx=0.1)
    sc.scheme.normal_pred_order = 0
    out.append(("rs_ctu", sc))
    sc = S.slip_weakening(nx=64, ny=32, dx=0.1)
    sc.scheme.use_prim_limiting = 0
    out.append(("sw_unlimited", sc))
    # PLM normal predictor: fourth-order slopes with primitive limiting (the decks'
    # slope setting), second-order slopes, characteristic limiting, no limiting
    for name, prim, char, fourth in (("rs_plm4", 1, 0, 1), ("sw_plm2", 1, 0, 0), ("sw_plm4_char", 0, 1, 1),
                                     ("rs_plm4_unlimited", 0, 0, 1)):
        sc = S.rate_state(nx=64, ny=32, dx=0.1) if name.startswith("rs") else S.slip_weakening(nx=64, ny=32, dx=0.1)
        sc.scheme.normal_pred_order = 1
        sc.scheme.use_prim_limiting, sc.scheme.use_char_limiting = prim, char
        sc.scheme.use_fourth_order_slopes = fourth
        out.append((name, sc))
    return out


SCEN = _scenarios()


def _random_B(sc, rng, n):
    B = sc.initial_B(xlo=0, xhi=n - 1 - 2 * A.TMK_NGHOST)
    if sc.scheme.fault_law == A.TMK_FAULT_RS:
        B[10] += 0.02 * rng.standard_normal(B.shape[1])
        B[8] = np.abs(rng.standard_normal(B.shape[1]))
    else:
        B[7] = 0.3 * np.abs(rng.standard_normal(B.shape[1]))
    return B


@pytest.mark.parametrize("name,sc", SCEN, ids=[n for n, _ in SCEN])
@pytest.mark.parametrize("valid", [(0, 0, 63, 31), (5, 0, 40, 13), (17, 9, 63, 31), (0, 3, 30, 31)],
                         ids=["whole", "fault_edge", "corner_hi", "edge_lo"])
def test_patch_update_state_matches_oracle(cuda_lib, name, sc, valid):
    import torch
    from tetemoko_gb300.level import Context, LinElastPatchGodunov
    rng = np.random.default_rng(1234)
    g = A.TMK_NGHOST
    ulo = (valid[0] - g, valid[1] - g)
    U0 = perturbed_state(sc, rng, lo=valid[:2], hi=valid[2:])
    touches = valid[1] == 0
    B0 = _random_B(sc, rng, valid[2] - valid[0] + 1 + 2 * g) if touches else None
    dt = sc.dt()
    time = 1.25
    # oracle
    Ur, Br = U0.copy(), (B0.copy() if B0 is not None else None)
    rc, Fxr, Fyr = O.patch_update_state(sc, Ur, ulo, valid[:2], valid[2:], Br, valid[0] - g, time, dt,
                                        with_flux=True)
    assert rc == 0
    # GPU
    ctx = Context(sc)
    pg = LinElastPatchGodunov(ctx)
    pg.set_current_box(valid)
    pg.set_current_time(time)
    Ud = torch.from_numpy(U0.copy()).cuda()
    Bd = torch.from_numpy(B0.copy()).cuda() if B0 is not None else None
    mws, Fx, Fy = pg.update_state(Ud, ulo, dt, B=Bd, bxlo=valid[0] - g, with_flux=True)
    torch.cuda.synchronize()
    assert mws == max(sc.elastic.cs, sc.elastic.cp)
    Ug = Ud.cpu().numpy()
    vs = (slice(None), slice(g, -g), slice(g, -g))
    assert rel_err(Ug[vs], Ur[vs]) <= RTOL_FP64
    # lambda, gamma and ghost cells are untouched
    assert np.array_equal(Ug[[9, 10, 20, 21]], U0[[9, 10, 20, 21]])
    assert np.array_equal(Ug[:, :g, :], U0[:, :g, :])
    ev = [c for c in range(22) if c % 11 < 9]
    assert rel_err(Fx.cpu().numpy()[ev], Fxr[ev]) <= RTOL_FP64
    assert rel_err(Fy.cpu().numpy()[ev], Fyr[ev]) <= RTOL_FP64
    if touches:
        Bg = Bd.cpu().numpy()
        bs = slice(g, -g)
        assert rel_err(Bg[:, bs], Br[:, bs]) <= RTOL_FP64
    ctx.close()


@pytest.mark.parametrize("name,sc", SCEN[:4], ids=[n for n, _ in SCEN[:4]])
def test_level_steps_match_oracle(cuda_lib, name, sc):
    """Ten steps of a level of uneven patches (exchange, fault row split across patches)."""
    from tetemoko_gb300.level import Context, LinElastLevelGodunov
    rng = np.random.default_rng(99)
    boxes = [(0, 0, 20, 9), (21, 0, 63, 9), (0, 10, 31, 31), (32, 10, 47, 20), (32, 21, 47, 31), (48, 10, 63, 31)]
    Ug = perturbed_state(sc, rng, amp_v=0.05, amp_s=1.0)
    Bg = sc.initial_B()
    Ur, Br = Ug.copy(), Bg.copy()
    ctx = Context(sc)
    lvl = LinElastLevelGodunov(ctx, boxes)
    lvl.set_level(Ug, Bg)
    dt = sc.dt()
    t = 0.0
    for n in range(10):
        assert O.level_step(sc, Ur, Br, boxes, t, dt) == 0
        lvl.step(t, dt)
        t += dt
    Uo, Bo = Ug.copy(), Bg.copy()
    lvl.get_level(Uo, Bo)
    g = A.TMK_NGHOST
    vs = (slice(None), slice(g, -g), slice(g, -g))
    assert rel_err(Uo[vs], Ur[vs]) <= 1e-11
    assert rel_err(Bo[:, g:-g], Br[:, g:-g]) <= 1e-11
    rc, info = lvl.status()
    assert rc == 0 and info[0] == 0
    lvl.close()
    ctx.close()


@pytest.mark.parametrize("prec", [A.TMK_PREC_FP64, A.TMK_PREC_MIXED], ids=["fp64", "mixed"])
@pytest.mark.parametrize("plastic", [False, True], ids=["elastic", "plastic"])
def test_steps_through_valid_put_and_take_equal_device_steps(cuda_lib, prec, plastic):
    """A level whose state goes to host arrays and back every step through
    tmk_level_put_valid / tmk_level_take_valid (only what a step reads and
    rewrites) steps exactly as one whose state stays on the device; the
    components and ghost cells the calls leave alone are untouched."""
    import torch
    from tetemoko_gb300.level import Context, LinElastLevelGodunov
    boxes = [(0, 0, 20, 9), (21, 0, 63, 9), (0, 10, 31, 31), (32, 10, 63, 31)]
    if plastic:
        sc = S.slip_weakening(nx=64, ny=32, dx=0.1, precision=prec, plasticity=True)
    else:
        sc = S.rate_state(nx=64, ny=32, dx=0.1, precision=prec)
    rng = np.random.default_rng(17)
    Ug = perturbed_state(sc, rng, amp_v=0.05, amp_s=1.0)
    if plastic:
        for side in (0, 11):
            Ug[side + 6, 8:14, :] += 60.0
    Bg = sc.initial_B()
    dt = sc.dt()
    ctx = Context(sc)
    ref = LinElastLevelGodunov(ctx, boxes)
    ref.set_level(Ug, Bg)
    lvl = LinElastLevelGodunov(ctx, boxes)
    lvl.set_level(Ug, Bg)
    # per-patch host arrays (pinned, read in place, and pageable, staged)
    Us, Bs = [], []
    for p in range(len(boxes)):
        U, B = lvl.get_patch(p)
        if p % 2 == 0:
            U = torch.from_numpy(U).pin_memory().numpy()
        Us.append(U)
        Bs.append(B)
    U_before = [u.copy() for u in Us]
    for n in range(4):
        ref.step(n * dt, dt)
        for p in range(len(boxes)):
            lvl.put_valid(p, Us[p], Bs[p])
        lvl.step(n * dt, dt)
        for p in range(len(boxes)):
            lvl.take_valid(p, Us[p], Bs[p])
    torch.cuda.synchronize()
    g = A.TMK_NGHOST
    evolving = [c for c in range(22) if plastic or c % 11 < 9]
    other = [c for c in range(22) if c not in evolving]
    for p in range(len(boxes)):
        Ur, Br = ref.get_patch(p)
        vs = (evolving, slice(g, -g), slice(g, -g))
        np.testing.assert_array_equal(Us[p][:, g:-g, g:-g][evolving], Ur[:, g:-g, g:-g][evolving])
        if Bs[p] is not None:
            np.testing.assert_array_equal(Bs[p], Br)
        # untouched: the other components everywhere, every ghost cell
        np.testing.assert_array_equal(Us[p][other], U_before[p][other])
        ghost = np.ones(Us[p].shape[1:], dtype=bool)
        ghost[g:-g, g:-g] = False
        np.testing.assert_array_equal(Us[p][:, ghost], U_before[p][:, ghost])
    assert ref.status()[0] == 0 and lvl.status()[0] == 0
    ref.close()
    lvl.close()
    ctx.close()


def test_plastic_update_matches_oracle(cuda_lib):
    import torch
    from tetemoko_gb300.level import Context, LinElastPatchGodunov
    sc = S.slip_weakening(nx=32, ny=16, dx=0.1, plasticity=True)
    rng = np.random.default_rng(7)
    U0 = perturbed_state(sc, rng, amp_s=60.0)
    U0[[10, 21]] = np.abs(rng.standard_normal((2,) + U0.shape[1:]))
    g = A.TMK_NGHOST
    Ur = U0.copy()
    O.plastic_correction(sc, Ur, (-g, -g), (0, 0), (31, 15), sc.dt())
    ctx = Context(sc)
    pg = LinElastPatchGodunov(ctx)
    Ud = torch.from_numpy(U0.copy()).cuda()
    pg.plastic_update(Ud, (-g, -g), sc.dt(), box=(0, 0, 31, 15))
    Ug = Ud.cpu().numpy()
    assert (Ur[9] > 0).any(), "the test state must yield somewhere"
    assert rel_err(Ug, Ur) <= RTOL_FP64
    ctx.close()


@pytest.mark.parametrize("name", ["rs_slip", "rs_aging"])
def test_level_steps_with_per_face_friction_match_oracle(cuda_lib, name):
    """Per-face a, b, L (+-10% about the scenario's, seed 4001) on a level of
    uneven patches: ten steps against the oracle given the same field."""
    from tetemoko_gb300.level import Context, LinElastLevelGodunov
    sc = dict(SCEN)[name]
    rng = np.random.default_rng(98)
    boxes = [(0, 0, 20, 9), (21, 0, 63, 9), (0, 10, 31, 31), (32, 10, 63, 31)]
    Ug = perturbed_state(sc, rng, amp_v=0.05, amp_s=1.0)
    Bg = sc.initial_B()
    F = S.friction_field(sc, seed=4001)
    Ur, Br = Ug.copy(), Bg.copy()
    ctx = Context(sc)
    lvl = LinElastLevelGodunov(ctx, boxes)
    lvl.set_level(Ug, Bg)
    lvl.set_level_friction(F)
    dt = sc.dt()
    t = 0.0
    for n in range(10):
        assert O.level_step(sc, Ur, Br, boxes, t, dt, fric=F) == 0
        lvl.step(t, dt)
        t += dt
    Uo, Bo = Ug.copy(), Bg.copy()
    lvl.get_level(Uo, Bo)
    g = A.TMK_NGHOST
    assert rel_err(Uo[:, g:-g, g:-g], Ur[:, g:-g, g:-g]) <= 1e-11
    assert rel_err(Bo[:, g:-g], Br[:, g:-g]) <= 1e-11
    # the field mattered: the constant-friction oracle run differs
    Uc, Bc = Ug.copy(), Bg.copy()
    t = 0.0
    for n in range(10):
        assert O.level_step(sc, Uc, Bc, boxes, t, dt) == 0
        t += dt
    assert rel_err(Bc[10:11, g:-g], Br[10:11, g:-g]) > 1e-9
    rc, info = lvl.status()
    assert rc == 0 and info[0] == 0
    lvl.close()
    ctx.close()


def test_fault_friction_descriptor_checks(cuda_lib):
    from tetemoko_gb300.level import Context, LinElastLevelGodunov
    sc = S.rate_state(nx=64, ny=32, dx=0.1)
    ctx = Context(sc)
    lvl = LinElastLevelGodunov(ctx, [(0, 0, 63, 15), (0, 16, 63, 31)])
    F = S.friction_field(sc)
    with pytest.raises(A.TmkError):
        lvl.set_fault_friction(1, F)             # patch 1 is not on the fault
    F[1, 7] = 0.0
    with pytest.raises(A.TmkError):
        lvl.set_fault_friction(0, F)             # b must be positive
    lvl.close()
    ctx.close()
    sw = S.slip_weakening(nx=64, ny=32, dx=0.1)
    ctx = Context(sw)
    lvl = LinElastLevelGodunov(ctx, [(0, 0, 63, 31)])
    with pytest.raises(A.TmkError):
        lvl.set_fault_friction(0, S.friction_field(sc))   # slip weakening has no a, b, L
    lvl.close()
    ctx.close()


@pytest.mark.parametrize("name", ["rs_plm4", "sw_plm4_char"])
def test_plm_level_steps_match_oracle(cuda_lib, name):
    """Ten steps of a level of uneven patches with the PLM predictor (the tile
    volume kernel, the fault kernel's PLM predictors) against the oracle."""
    from tetemoko_gb300.level import Context, LinElastLevelGodunov
    sc = dict(SCEN)[name]
    rng = np.random.default_rng(97)
    boxes = [(0, 0, 20, 9), (21, 0, 63, 9), (0, 10, 31, 31), (32, 10, 63, 31)]
    Ug = perturbed_state(sc, rng, amp_v=0.05, amp_s=1.0)
    Bg = sc.initial_B()
    Ur, Br = Ug.copy(), Bg.copy()
    ctx = Context(sc)
    lvl = LinElastLevelGodunov(ctx, boxes)
    lvl.set_level(Ug, Bg)
    dt = sc.dt()
    for n in range(10):
        assert O.level_step(sc, Ur, Br, boxes, n * dt, dt) == 0
        lvl.step(n * dt, dt)
    Uo, Bo = Ug.copy(), Bg.copy()
    lvl.get_level(Uo, Bo)
    g = A.TMK_NGHOST
    assert rel_err(Uo[:, g:-g, g:-g], Ur[:, g:-g, g:-g]) <= 1e-11
    assert rel_err(Bo[:, g:-g], Br[:, g:-g]) <= 1e-11
    assert lvl.status()[0] == 0
    lvl.close()
    ctx.close()


@pytest.mark.parametrize("name", ["rs_slip", "sw_ref9"])
def test_patch_step_staged_by_tma_or_element_wise_is_the_same(cuda_lib, name):
    """The tile kernel stages each tile and its halo with one TMA tensor copy
    when the FAB's base and row pitch are 16-byte aligned, else element by
    element: a FAB one column wider (odd row pitch in FP64) takes the second
    path, and the step is the same bit for bit."""
    import torch
    from tetemoko_gb300.level import Context, LinElastPatchGodunov
    sc = dict(SCEN)[name]
    g = A.TMK_NGHOST
    valid = (5, 0, 40, 13)                      # 36 columns: a row of 44 FP64 values (16-byte pitch)
    ulo = (valid[0] - g, valid[1] - g)
    rng = np.random.default_rng(4321)
    U0 = perturbed_state(sc, rng, lo=valid[:2], hi=valid[2:])
    B0 = _random_B(sc, rng, valid[2] - valid[0] + 1 + 2 * g)
    U1 = np.concatenate([U0, U0[:, :, -1:]], axis=2)     # one more ghost column on the right
    assert U0.shape[2] * 8 % 16 == 0 and U1.shape[2] * 8 % 16 != 0
    ctx = Context(sc)
    out = []
    for U in (U0, U1):
        pg = LinElastPatchGodunov(ctx)
        pg.set_current_box(valid)
        pg.set_current_time(0.5)
        Ud = torch.from_numpy(np.ascontiguousarray(U)).cuda()
        Bd = torch.from_numpy(B0.copy()).cuda()
        _, Fx, Fy = pg.update_state(Ud, ulo, sc.dt(), B=Bd, bxlo=valid[0] - g, with_flux=True)
        torch.cuda.synchronize()
        out.append((Ud.cpu().numpy()[:, :, :U0.shape[2]], Bd.cpu().numpy(), Fx.cpu().numpy(), Fy.cpu().numpy()))
    for a, b in zip(*out):
        np.testing.assert_array_equal(a, b)
    ctx.close()
