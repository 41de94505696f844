"""3-D patch step (CH_SPACEDIM == 3) on the GPU == the oracle's 3-D
restatement, through the C ABI (tmk_patch_update_state_3d,
tmk_plastic_update_3d).  FP64 on both sides: 1e-12 relative per component
(RTOL_FP64), for the state over the valid box, the face fluxes and the fault's
boundary data, on patches that touch the fault plane and the domain's edges in
every direction and on interior patches."""
import numpy as np
import pytest

import oracle as O
from tetemoko_gb300 import _capi as A, scenarios as S
from tests.helpers import RTOL_FP64, perturbed_state_3d, random_B_3d, rel_err

pytestmark = pytest.mark.gpu

G = A.TMK_NGHOST
NX, NY, NZ, DX = 12, 10, 8, 0.1
DOM = ((0, 0, 0), (NX - 1, NY - 1, NZ - 1))


def _sw(layout=A.TMK_SW_LAYOUT_OFFSET11):
    """Slip weakening with z profiles that vary over the test domain: a smooth
    nucleation patch centred at z = 0.4 and a friction box |z| < 0.5."""
    sc = S.slip_weakening(nx=NX, ny=NY, dx=DX, layout=layout)
    w = sc.sw
    w.smooth = 0.3
    w.xc[0], w.xw[0], w.zc[0], w.zw[0] = 0.1, 0.2, 0.4, 0.15
    w.num_patches = 2
    w.xc[1], w.xw[1], w.zc[1], w.zw[1], w.tau[1] = -0.3, 0.1, 0.1, 0.05, 4.0
    w.fric_box_width[0], w.fric_box_width[1] = 0.45, 0.5
    w.outside_friction = 2.0
    return sc


def _scenarios():
    out = []
    sc = S.rate_state(nx=NX, ny=NY, dx=DX, state_law=A.TMK_RS_SLIP_LAW)
    sc.rs.L = 0.5
    out.append(("rs_slip", sc))
    out.append(("rs_aging", S.rate_state(nx=NX, ny=NY, dx=DX)))
    out.append(("sw_ref9", _sw(A.TMK_SW_LAYOUT_REFERENCE9)))
    out.append(("sw_off11", _sw()))
    sc = _sw()
    sc.scheme.use_prim_limiting, sc.scheme.use_char_limiting = 0, 1
    out.append(("sw_charlim", sc))
    sc = S.rate_state(nx=NX, ny=NY, dx=DX)
    for k, v in enumerate((1, 0, 2, 1, 1, 0)):
        sc.scheme.boundary_type[k] = v
    out.append(("rs_free_edges", sc))
    sc = S.rate_state(nx=NX, ny=NY, dx=DX)
    sc.scheme.normal_pred_order = 0
    out.append(("rs_ctu", sc))
    sc = _sw()
    sc.scheme.normal_pred_order = 1
    out.append(("sw_plm4", sc))
    sc = S.rate_state(nx=NX, ny=NY, dx=DX)
    sc.scheme.normal_pred_order = 1
    sc.scheme.use_fourth_order_slopes = 0
    out.append(("rs_plm2", sc))
    sc = S.rate_state(nx=NX, ny=NY, dx=DX)
    sc.scheme.fault_law = A.TMK_FAULT_NONE
    for k, v in enumerate((0, 1, 0, 1, 1, 0)):
        sc.scheme.boundary_type[k] = v
    out.append(("no_fault", sc))
    return out


SCEN = _scenarios()
VALID = [((0, 0, 0), (11, 9, 7)), ((2, 0, 1), (9, 5, 6)), ((5, 4, 3), (11, 9, 7)), ((0, 3, 0), (7, 9, 4)),
         ((3, 2, 2), (8, 7, 5))]
VALID_IDS = ["whole", "fault_inner", "corner_hi", "edge_lo", "interior"]


@pytest.mark.parametrize("name,sc", SCEN, ids=[n for n, _ in SCEN])
@pytest.mark.parametrize("valid", VALID, ids=VALID_IDS)
def test_patch_update_state_3d_matches_oracle(cuda_lib, name, sc, valid):
    import torch
    from tetemoko_gb300.level import Context, LinElastPatchGodunov3D
    lo, hi = valid
    rng = np.random.default_rng(4321)
    U0 = perturbed_state_3d(sc, rng, lo, hi)
    ulo = tuple(l - G for l in lo)
    fault = sc.scheme.fault_law != A.TMK_FAULT_NONE and lo[1] == 0
    # fault data over the valid x, z grown by the ghost width
    blo = (lo[0] - G, lo[2] - G)
    B0 = random_B_3d(sc, rng, hi[0] - lo[0] + 1 + 2 * G, hi[2] - lo[2] + 1 + 2 * G) if fault else None
    dt, time = sc.dt(), 0.75
    Ur, Br = U0.copy(), (B0.copy() if fault else None)
    rc, Fr = O.patch_update_state_3d(sc, Ur, ulo, lo, hi, DOM[0], DOM[1], Br, blo, DX, time, dt, with_flux=True)
    assert rc == 0
    ctx = Context(sc)
    pg = LinElastPatchGodunov3D(ctx, DOM)
    pg.set_current_box(valid)
    pg.set_current_time(time)
    Ud = torch.from_numpy(U0.copy()).cuda()
    Bd = torch.from_numpy(B0.copy()).cuda() if fault else None
    mws, F = pg.update_state(Ud, ulo, dt, B=Bd, blo=blo, with_flux=True)
    torch.cuda.synchronize()
    assert mws == max(sc.elastic.cs, sc.elastic.cp)
    Ug = Ud.cpu().numpy()
    v = (slice(None), slice(G, -G), slice(G, -G), slice(G, -G))
    assert rel_err(Ug[v], Ur[v]) <= RTOL_FP64
    assert np.array_equal(Ug[[9, 10, 20, 21]], U0[[9, 10, 20, 21]])
    assert np.array_equal(Ug[:, :G], U0[:, :G])
    assert np.array_equal(Ug[:, :, :G], U0[:, :, :G])
    ev = [c for c in range(22) if c % 11 < 9]
    for d in range(3):
        assert rel_err(F[d].cpu().numpy()[ev], Fr[d][ev]) <= RTOL_FP64, d
    if fault:
        Bg = Bd.cpu().numpy()
        bv = (slice(None), slice(G, -G), slice(G, -G))
        assert rel_err(Bg[bv], Br[bv]) <= RTOL_FP64
        assert not np.array_equal(Br[bv], B0[bv])
    ctx.close()


def test_z_uniform_gpu_step_reduces_to_2d_gpu_step(cuda_lib):
    """A state without z variation on a patch away from the z edges: the 3-D
    kernels reproduce the 2-D patch kernels exactly off the fault row."""
    import torch
    from tetemoko_gb300.level import Context, LinElastPatchGodunov, LinElastPatchGodunov3D
    from tests.helpers import perturbed_state
    sc = S.rate_state(nx=NX, ny=NY, dx=DX)
    rng = np.random.default_rng(5)
    U2 = perturbed_state(sc, rng)
    B2 = sc.initial_B()
    ctx = Context(sc)
    p2 = LinElastPatchGodunov(ctx)
    p2.set_current_box((0, 0, NX - 1, NY - 1))
    U2d = torch.from_numpy(U2.copy()).cuda()
    p2.update_state(U2d, (-G, -G), sc.dt(), B=torch.from_numpy(B2.copy()).cuda(), bxlo=-G)
    p3 = LinElastPatchGodunov3D(ctx, ((0, 0, 0), (NX - 1, NY - 1, 9)))
    p3.set_current_box(((0, 0, 3), (NX - 1, NY - 1, 5)))
    U3 = torch.from_numpy(np.repeat(U2[:, None], 3 + 2 * G, axis=1).copy()).cuda()
    B3 = torch.from_numpy(np.repeat(B2[:, None], 3 + 2 * G, axis=1).copy()).cuda()
    p3.update_state(U3, (-G, -G, 3 - G), sc.dt(), B=B3, blo=(-G, 3 - G))
    torch.cuda.synchronize()
    a = U3.cpu().numpy()
    b = U2d.cpu().numpy()
    for k in range(G, G + 3):
        assert np.array_equal(a[:, k, G + 1:], b[:, G + 1:])
    ctx.close()


def test_plastic_update_3d_matches_oracle(cuda_lib):
    import torch
    from tetemoko_gb300.level import Context, LinElastPatchGodunov3D
    sc = S.slip_weakening(nx=NX, ny=NY, dx=DX, plasticity=True)
    rng = np.random.default_rng(8)
    lo, hi = (0, 0, 0), (NX - 1, NY - 1, NZ - 1)
    U0 = perturbed_state_3d(sc, rng, lo, hi, amp_s=60.0)
    U0[[10, 21]] = np.abs(rng.standard_normal((2,) + U0.shape[1:]))
    Ur = U0.copy()
    box = ((1, 0, 2), (10, 8, 7))
    O.plastic_correction_3d(sc, Ur, (-G, -G, -G), box[0], box[1], sc.dt())
    ctx = Context(sc)
    pg = LinElastPatchGodunov3D(ctx, DOM)
    Ud = torch.from_numpy(U0.copy()).cuda()
    pg.plastic_update(Ud, (-G, -G, -G), sc.dt(), box=box)
    Ug = Ud.cpu().numpy()
    assert (Ur[9] > 0).any(), "the test state must yield somewhere"
    assert rel_err(Ug, Ur) <= RTOL_FP64
    ctx.close()


def test_bad_descriptors_are_refused(cuda_lib):
    import torch
    from tetemoko_gb300.level import Context, LinElastPatchGodunov3D
    sc = S.rate_state(nx=NX, ny=NY, dx=DX)
    ctx = Context(sc)
    pg = LinElastPatchGodunov3D(ctx, DOM)
    pg.set_current_box(((0, 1, 0), (5, 5, 5)))
    U = torch.zeros((22, 6 + 2, 5 + 2, 6 + 2), dtype=torch.float64, device="cuda")   # too few ghosts
    with pytest.raises(A.TmkError):
        pg.update_state(U, (-1, 0, -1), sc.dt())
    pg.set_current_box(((0, 0, 0), (5, 5, 5)))
    U = torch.zeros((22, 6 + 2 * G, 6 + 2 * G, 6 + 2 * G), dtype=torch.float64, device="cuda")
    with pytest.raises(A.TmkError):      # a fault patch without fault data
        pg.update_state(U, (-G, -G, -G), sc.dt())
    ctx.close()


MIXED = [n for n in ("rs_slip", "rs_aging", "sw_ref9", "sw_off11", "sw_charlim", "rs_plm2", "rs_ctu", "no_fault")]


@pytest.mark.parametrize("name", MIXED)
def test_mixed_patch_step_3d_close_to_oracle(cuda_lib, name):
    """The mixed form (FP32 volume arithmetic and intermediates; FP64 state,
    friction and boundary data) against the FP64 oracle: one step, FP32
    rounding of the increments (2e-5 of each component's scale for the state
    and the fluxes, 1e-3 for the fault's boundary data, whose slip rates
    amplify the rounding of the shear through the friction law)."""
    import torch
    from tetemoko_gb300.level import Context, LinElastPatchGodunov3D
    sc = dict(SCEN)[name]
    lo, hi = (0, 0, 0), (NX - 1, NY - 1, NZ - 1)
    rng = np.random.default_rng(77)
    U0 = perturbed_state_3d(sc, rng, lo, hi)
    fault = sc.scheme.fault_law != A.TMK_FAULT_NONE
    blo = (-G, -G)
    B0 = random_B_3d(sc, rng, NX + 2 * G, NZ + 2 * G) if fault else None
    dt, time = sc.dt(), 0.5
    Ur, Br = U0.copy(), (B0.copy() if fault else None)
    rc, Fr = O.patch_update_state_3d(sc, Ur, (-G, -G, -G), lo, hi, DOM[0], DOM[1], Br, blo, DX, time, dt,
                                     with_flux=True)
    assert rc == 0
    old = sc.scheme.precision
    sc.scheme.precision = A.TMK_PREC_MIXED
    try:
        ctx = Context(sc)
    finally:
        sc.scheme.precision = old
    pg = LinElastPatchGodunov3D(ctx, DOM)
    pg.set_current_box((lo, hi))
    pg.set_current_time(time)
    Ud = torch.from_numpy(U0.copy()).cuda()
    Bd = torch.from_numpy(B0.copy()).cuda() if fault else None
    _, F = pg.update_state(Ud, (-G, -G, -G), dt, B=Bd, blo=blo, with_flux=True)
    torch.cuda.synchronize()
    Ug = Ud.cpu().numpy()
    v = (slice(None), slice(G, -G), slice(G, -G), slice(G, -G))
    eu = rel_err(Ug[v], Ur[v])
    ev = [c for c in range(22) if c % 11 < 9]
    ef = max(rel_err(F[d].cpu().numpy()[ev], Fr[d][ev]) for d in range(3))
    print(name, "state", eu, "flux", ef)
    assert eu < 2e-5 and ef < 2e-5
    assert eu > 0.0, "the mixed form must not be the FP64 path"
    if fault:
        bv = (slice(None), slice(G, -G), slice(G, -G))
        eb = rel_err(Bd.cpu().numpy()[bv], Br[bv])
        print(name, "bdry", eb)
        assert eb < 1e-3
    ctx.close()


def test_mixed_3d_tracks_fp64_over_steps(cuda_lib):
    """Twenty steps of a smooth rate-and-state state in both forms on the GPU:
    the mixed form stays within 1e-4 of the FP64 form."""
    import torch
    from tetemoko_gb300.level import Context, LinElastPatchGodunov3D
    sc = S.rate_state(nx=NX, ny=NY, dx=DX)
    lo, hi = (0, 0, 0), (NX - 1, NY - 1, NZ - 1)
    rng = np.random.default_rng(12)
    U0 = perturbed_state_3d(sc, rng, lo, hi, amp_v=0.01, amp_s=0.5)
    B0 = random_B_3d(sc, rng, NX + 2 * G, NZ + 2 * G)
    out = {}
    for prec in (A.TMK_PREC_FP64, A.TMK_PREC_MIXED):
        sc.scheme.precision = prec
        ctx = Context(sc)
        pg = LinElastPatchGodunov3D(ctx, DOM)
        pg.set_current_box((lo, hi))
        Ud = torch.from_numpy(U0.copy()).cuda()
        Bd = torch.from_numpy(B0.copy()).cuda()
        for n in range(20):
            pg.set_current_time(n * sc.dt())
            pg.update_state(Ud, (-G, -G, -G), sc.dt(), B=Bd, blo=(-G, -G))
        torch.cuda.synchronize()
        out[prec] = (Ud.cpu().numpy(), Bd.cpu().numpy())
        ctx.close()
    sc.scheme.precision = A.TMK_PREC_FP64
    v = (slice(None), slice(G, -G), slice(G, -G), slice(G, -G))
    a, b = out[A.TMK_PREC_MIXED][0][v], out[A.TMK_PREC_FP64][0][v]
    assert np.isfinite(a).all()
    e = rel_err(a, b)
    print("20 steps", e)
    assert 0.0 < e < 1e-4


TILES = [((0, 0, 0), (5, 4, 7)), ((6, 0, 0), (11, 4, 3)), ((6, 0, 4), (11, 4, 7)), ((0, 5, 0), (11, 9, 7))]


@pytest.mark.parametrize("name", ["rs_aging", "sw_ref9", "no_fault"])
@pytest.mark.parametrize("prec", [A.TMK_PREC_FP64, A.TMK_PREC_MIXED], ids=["fp64", "mixed"])
def test_batched_patches_equal_the_whole_domain_step(cuda_lib, name, prec):
    """tmk_patches_update_state_3d on patches tiling the domain (ghosts taken
    from the same global state, as an exchange leaves them) gives bit for bit
    the step of one patch over the whole domain, and the same as one call per
    patch.  In the mixed form the FP64 boundary-data update is built with FMA
    contraction, which the compiler may apply differently in the single-patch
    and batched kernels (a*a + b*b fused either way): there the boundary data
    agree to 1e-12."""
    import torch
    from tetemoko_gb300.level import Context, LinElastPatchGodunov3D
    sc = dict(SCEN)[name]
    rng = np.random.default_rng(99)
    lo, hi = (0, 0, 0), (NX - 1, NY - 1, NZ - 1)
    U0 = perturbed_state_3d(sc, rng, lo, hi)
    fault = sc.scheme.fault_law != A.TMK_FAULT_NONE
    B0 = random_B_3d(sc, rng, NX + 2 * G, NZ + 2 * G) if fault else None
    old = sc.scheme.precision
    sc.scheme.precision = prec
    try:
        ctx = Context(sc)
    finally:
        sc.scheme.precision = old
    dt, time = sc.dt(), 0.5
    pg = LinElastPatchGodunov3D(ctx, DOM)
    pg.set_current_time(time)
    # the whole domain as one patch
    Uw = torch.from_numpy(U0.copy()).cuda()
    Bw = torch.from_numpy(B0.copy()).cuda() if fault else None
    pg.set_current_box((lo, hi))
    pg.update_state(Uw, (-G, -G, -G), dt, B=Bw, blo=(-G, -G))

    def tile_arrays(v):
        (l0, l1, l2), (h0, h1, h2) = v
        U = torch.from_numpy(np.ascontiguousarray(U0[:, l2:h2 + 2 * G + 1, l1:h1 + 2 * G + 1, l0:h0 + 2 * G + 1])).cuda()
        B = None
        if fault and l1 == 0:
            B = torch.from_numpy(np.ascontiguousarray(B0[:, l2:h2 + 2 * G + 1, l0:h0 + 2 * G + 1])).cuda()
        return U, (l0 - G, l1 - G, l2 - G), B, (l0 - G, l2 - G)

    batch = []
    single = []
    for v in TILES:
        U, ulo, B, blo = tile_arrays(v)
        batch.append((v, U, ulo, B, blo))
        U2, _, B2, _ = tile_arrays(v)
        pg.set_current_box(v)
        pg.update_state(U2, ulo, dt, B=B2, blo=blo)
        single.append((U2, B2))
    pg.update_states(batch, dt)
    torch.cuda.synchronize()
    Uwh = Uw.cpu().numpy()
    Bwh = Bw.cpu().numpy() if fault else None
    for (v, U, ulo, B, blo), (U2, B2) in zip(batch, single):
        (l0, l1, l2), (h0, h1, h2) = v
        a = U.cpu().numpy()[:, G:-G, G:-G, G:-G]
        np.testing.assert_array_equal(a, U2.cpu().numpy()[:, G:-G, G:-G, G:-G])
        np.testing.assert_array_equal(a, Uwh[:, l2 + G:h2 + G + 1, l1 + G:h1 + G + 1, l0 + G:h0 + G + 1])
        if B is not None:
            b = B.cpu().numpy()[:, G:-G, G:-G]
            for ref in (B2.cpu().numpy()[:, G:-G, G:-G], Bwh[:, l2 + G:h2 + G + 1, l0 + G:h0 + G + 1]):
                if prec == A.TMK_PREC_FP64:
                    np.testing.assert_array_equal(b, ref)
                else:
                    assert rel_err(b, ref) <= 1e-12
    ctx.close()


def _run_rupture_3d(sc, nz, nsteps, stations, kmid):
    """A z-uniform rate-and-state nucleation on one 3-D patch (outflow z
    faces): fault slip-rate history at the stations of row kmid, and the final
    state and fault data."""
    import torch
    from tetemoko_gb300.level import Context, LinElastPatchGodunov3D
    nx, ny = sc.nx, sc.ny
    lo, hi = (0, 0, 0), (nx - 1, ny - 1, nz - 1)
    U0 = np.empty((22, nz + 2 * G, ny + 2 * G, nx + 2 * G))
    U0[:] = sc.background()[:, None, None, None]
    B0 = np.ascontiguousarray(np.repeat(sc.initial_B()[:, None, :], nz + 2 * G, axis=1))
    ctx = Context(sc)
    pg = LinElastPatchGodunov3D(ctx, (lo, hi))
    pg.set_current_box((lo, hi))
    U = torch.from_numpy(U0).cuda()
    B = torch.from_numpy(B0).cuda()
    dt, t = sc.dt() / 3 ** 0.5, 0.0
    idx = torch.tensor([i + G for i in stations], device="cuda")
    hist, ts = [], []
    for _ in range(nsteps):
        pg.set_current_time(t)
        pg.update_state(U, (-G, -G, -G), dt, B=B, blo=(-G, -G))
        t += dt
        hist.append(B[2, kmid + G].index_select(0, idx).clone())
        ts.append(t)
    torch.cuda.synchronize()
    out = (np.array(ts), torch.stack(hist).cpu().numpy(), U.cpu().numpy(), B.cpu().numpy())
    ctx.close()
    return out


def test_mixed_3d_rupture_metrics_vs_fp64(cuda_lib):
    """The 3-D mixed form through nucleation and rupture against the 3-D FP64
    form (equal to the oracle per step): rupture arrival at fault stations 2-6 km
    either side of the nucleation (0.5 %), final slip (1e-3), peak slip rate
    (1e-2) and the particle velocities of the volume (1e-2), as the 2-D mixed
    form's rupture test."""
    from tests.test_gpu_mixed import _arrival
    nz, nsteps = 8, 450
    sc64 = S.rate_state(nx=192, ny=64, dx=0.1)
    scm = S.rate_state(nx=192, ny=64, dx=0.1, precision=A.TMK_PREC_MIXED)
    x0 = sc64.rs.x0
    st = [int(round((x0 + s * d) / sc64.dx - 0.5)) for d in (2.0, 4.0, 6.0) for s in (-1, 1)]
    kmid = nz // 2
    tr, Vr, Ur, Br = _run_rupture_3d(sc64, nz, nsteps, st, kmid)
    tm, Vm, Um, Bm = _run_rupture_3d(scm, nz, nsteps, st, kmid)
    thr = sc64.rs.rupture_threshold
    ar, am = _arrival(tr, Vr, thr), _arrival(tm, Vm, thr)
    assert np.all(np.isfinite(ar)), "every station must rupture within the run"
    arr_err = np.max(np.abs(am - ar) / ar)
    sl = [i + G for i in st]
    slip_r, slip_m = Br[8, kmid + G, sl], Bm[8, kmid + G, sl]
    slip_err = np.max(np.abs(slip_m - slip_r) / np.abs(slip_r))
    peak_err = np.max(np.abs(Vm.max(axis=0) - Vr.max(axis=0)) / Vr.max(axis=0))
    vcomp = [0, 1, 2, 11, 12, 13]
    vs = (vcomp, slice(G, -G), slice(G, -G), slice(G, -G))
    vel_err = np.abs(Um[vs] - Ur[vs]).max() / np.abs(Ur[vs]).max()
    print(f"3-D mixed vs FP64: arrival {arr_err:.2e}, final slip {slip_err:.2e}, "
          f"peak slip rate {peak_err:.2e}, volume velocity {vel_err:.2e}")
    assert arr_err < 5e-3
    assert slip_err < 1e-3
    assert peak_err < 1e-2
    assert vel_err < 1e-2


# The device 3-D level (tmk_level3d): its step (device ghost exchange, the
# batched patch loop, the plastic correction on plastic schemes) over patches
# tiling the domain, from ghosts set as any values, equals steps of one patch
# over the whole domain.
LEVEL_TILINGS = {
    "regular": [((x0, y0, z0), (x0 + 5, y0 + 4, z0 + 3)) for z0 in (0, 4) for y0 in (0, 5) for x0 in (0, 6)],
    "uneven": [((0, 0, 0), (4, 9, 7)), ((5, 0, 0), (11, 2, 7)), ((5, 3, 0), (11, 9, 2)), ((5, 3, 3), (11, 9, 7))],
}


def _level3d_vs_whole(sc, tiles, prec, nsteps, amp_s=5.0):
    """(whole-domain U, B; level U, B per patch) after nsteps from one perturbed
    state; the level's patches start with their ghost cells set to NaN, which
    the exchange must overwrite inside the domain (the step reads no ghost
    outside it)."""
    import torch
    from tetemoko_gb300.level import Context, LinElastLevelGodunov3D, LinElastPatchGodunov3D
    rng = np.random.default_rng(123)
    lo, hi = DOM
    U0 = perturbed_state_3d(sc, rng, lo, hi, amp_s=amp_s)
    fault = sc.scheme.fault_law != A.TMK_FAULT_NONE
    B0 = random_B_3d(sc, rng, NX + 2 * G, NZ + 2 * G) if fault else None
    old = sc.scheme.precision
    sc.scheme.precision = prec
    try:
        ctx = Context(sc)
    finally:
        sc.scheme.precision = old
    dt, t0 = sc.dt() / 3 ** 0.5, 0.5
    pg = LinElastPatchGodunov3D(ctx, DOM)
    pg.set_current_box(DOM)
    Uw = torch.from_numpy(U0.copy()).cuda()
    Bw = torch.from_numpy(B0.copy()).cuda() if fault else None
    for k in range(nsteps):
        pg.set_current_time(t0 + k * dt)
        pg.update_state(Uw, (-G, -G, -G), dt, B=Bw, blo=(-G, -G))
        if sc.scheme.plasticity:
            pg.plastic_update(Uw, (-G, -G, -G), dt, box=DOM)
    lvl = LinElastLevelGodunov3D(ctx, tiles, DOM)
    for p, ((l0, l1, l2), (h0, h1, h2)) in enumerate(tiles):
        U = np.full(lvl.patch_shapes(p)[0], np.nan)
        U[:, G:-G, G:-G, G:-G] = U0[:, l2 + G:h2 + G + 1, l1 + G:h1 + G + 1, l0 + G:h0 + G + 1]
        B = None
        if lvl.touches_fault(p):
            B = np.full(lvl.patch_shapes(p)[1], np.nan)
            B[:, G:-G, G:-G] = B0[:, l2 + G:h2 + G + 1, l0 + G:h0 + G + 1]
        lvl.set_patch(p, U, B)
    for k in range(nsteps):
        lvl.step(t0 + k * dt, dt)
    got = [lvl.get_patch(p) for p in range(len(tiles))]
    torch.cuda.synchronize()
    out = (Uw.cpu().numpy(), Bw.cpu().numpy() if fault else None, got)
    lvl.close()
    ctx.close()
    return out


@pytest.mark.parametrize("name", ["rs_aging", "sw_off11", "no_fault"])
@pytest.mark.parametrize("tiling", list(LEVEL_TILINGS))
@pytest.mark.parametrize("prec", [A.TMK_PREC_FP64, A.TMK_PREC_MIXED], ids=["fp64", "mixed"])
def test_level3d_steps_equal_whole_domain_steps(cuda_lib, name, tiling, prec):
    """Three level steps: the FP64 form bit for bit; the mixed form to 1e-10
    (its boundary-data update may contract a product differently in the
    single-patch and batched kernels, and the fault data feed the state)."""
    sc = dict(SCEN)[name]
    tiles = LEVEL_TILINGS[tiling]
    Uw, Bw, got = _level3d_vs_whole(sc, tiles, prec, 3)
    for ((l0, l1, l2), (h0, h1, h2)), (U, B) in zip(tiles, got):
        a = U[:, G:-G, G:-G, G:-G]
        ref = Uw[:, l2 + G:h2 + G + 1, l1 + G:h1 + G + 1, l0 + G:h0 + G + 1]
        if prec == A.TMK_PREC_FP64:
            np.testing.assert_array_equal(a, ref)
        else:
            assert rel_err(a, ref) <= 1e-10
        if B is not None:
            b, bref = B[:, G:-G, G:-G], Bw[:, l2 + G:h2 + G + 1, l0 + G:h0 + G + 1]
            if prec == A.TMK_PREC_FP64:
                np.testing.assert_array_equal(b, bref)
            else:
                assert rel_err(b, bref) <= 1e-10


def test_level3d_plastic_steps_equal_whole_domain_steps(cuda_lib):
    """A plastic slip-weakening level (stresses large enough to yield): the
    level applies the plastic correction after each step, as one patch over
    the whole domain does (FP64, bit for bit)."""
    sc = S.slip_weakening(nx=NX, ny=NY, dx=DX, plasticity=True)
    tiles = LEVEL_TILINGS["uneven"]
    Uw, Bw, got = _level3d_vs_whole(sc, tiles, A.TMK_PREC_FP64, 3, amp_s=60.0)
    yielded = 0
    for ((l0, l1, l2), (h0, h1, h2)), (U, B) in zip(tiles, got):
        ref = Uw[:, l2 + G:h2 + G + 1, l1 + G:h1 + G + 1, l0 + G:h0 + G + 1]
        np.testing.assert_array_equal(U[:, G:-G, G:-G, G:-G], ref)
        yielded += int(np.count_nonzero(ref[9]))
    assert yielded > 0, "no cell yielded: the plastic correction was not exercised"


def test_level3d_rejects_overlapping_or_outside_boxes(cuda_lib):
    from tetemoko_gb300.level import Context, LinElastLevelGodunov3D
    sc = dict(SCEN)["rs_aging"]
    ctx = Context(sc)
    for boxes in ([((0, 0, 0), (6, 9, 7)), ((6, 0, 0), (11, 9, 7))],       # overlap at x = 6
                  [((0, 0, 0), (12, 9, 7))]):                               # beyond the domain in x
        with pytest.raises(RuntimeError):
            LinElastLevelGodunov3D(ctx, boxes, DOM)
    ctx.close()
