"""The column-marching volume kernel equals the oracle (FP64 instantiation, 1e-12)
and the tile kernel (FP32 instantiation, FP32 rounding) on multi-patch levels."""
import numpy as np
import pytest

import oracle as O
from tetemoko_gb300 import _capi as A, scenarios as S
from tests.helpers import perturbed_state, rel_err

pytestmark = pytest.mark.gpu

BOXES = [(0, 0, 20, 9), (21, 0, 63, 9), (0, 10, 31, 31), (32, 10, 47, 20), (32, 21, 47, 31), (48, 10, 63, 31)]


def _cases():
    out = []
    sc = S.rate_state(nx=64, ny=32, dx=0.1, state_law=A.TMK_RS_SLIP_LAW)
    sc.rs.L = 0.5
    out.append(("rs_slip", sc))
    out.append(("rs_aging", S.rate_state(nx=64, ny=32, dx=0.1)))
    out.append(("sw_ref9", S.slip_weakening(nx=64, ny=32, dx=0.1, layout=A.TMK_SW_LAYOUT_REFERENCE9)))
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
    return out


CASES = _cases()


def _run_level(sc, boxes, U0, B0, nsteps, info_out=None):
    from tetemoko_gb300.level import Context, LinElastLevelGodunov
    ctx = Context(sc)
    lvl = LinElastLevelGodunov(ctx, boxes)
    lvl.set_level(U0, B0)
    t = 0.0
    for _ in range(nsteps):
        lvl.step(t, sc.dt())
        t += sc.dt()
    U, B = U0.copy(), B0.copy()
    lvl.get_level(U, B)
    rc, info = lvl.status()
    lvl.close()
    ctx.close()
    assert rc == 0, info
    if info_out is not None:
        info_out.extend(info)
    return U, B


@pytest.mark.parametrize("name,sc", CASES, ids=[n for n, _ in CASES])
@pytest.mark.parametrize("boxes", [BOXES, [(0, 0, 63, 31)]], ids=["six_patches", "one_patch"])
def test_march_fp64_matches_oracle(cuda_lib, name, sc, boxes):
    sc.scheme.volume_kernel = A.TMK_VOLUME_MARCH
    rng = np.random.default_rng(5)
    U0 = perturbed_state(sc, rng, amp_v=0.05, amp_s=1.0)
    B0 = sc.initial_B()
    Ur, Br = U0.copy(), B0.copy()
    t = 0.0
    for _ in range(6):
        assert O.level_step(sc, Ur, Br, boxes, t, sc.dt()) == 0
        t += sc.dt()
    Ug, Bg = _run_level(sc, boxes, U0, B0, 6)
    g = A.TMK_NGHOST
    vs = (slice(None), slice(g, -g), slice(g, -g))
    assert rel_err(Ug[vs], Ur[vs]) <= 1e-11
    assert rel_err(Bg[:, g:-g], Br[:, g:-g]) <= 1e-11


@pytest.mark.parametrize("name,sc", CASES[:3], ids=[n for n, _ in CASES[:3]])
def test_march_fp32_is_as_accurate_as_tile_fp32(cuda_lib, name, sc):
    """Both FP32 volume kernels round differently; each is measured against the
    FP64 oracle and the marching kernel must be about as accurate."""
    rng = np.random.default_rng(6)
    U0 = perturbed_state(sc, rng, amp_v=0.05, amp_s=1.0)
    B0 = sc.initial_B()
    Ur, Br = U0.copy(), B0.copy()
    t = 0.0
    for _ in range(6):
        assert O.level_step(sc, Ur, Br, BOXES, t, sc.dt()) == 0
        t += sc.dt()
    sc.scheme.precision = A.TMK_PREC_MIXED
    sc.scheme.volume_kernel = A.TMK_VOLUME_TILE
    Ut, Bt = _run_level(sc, BOXES, U0, B0, 6)
    sc.scheme.volume_kernel = A.TMK_VOLUME_MARCH
    Um, Bm = _run_level(sc, BOXES, U0, B0, 6)
    g = A.TMK_NGHOST
    vs = (slice(None), slice(g, -g), slice(g, -g))
    et, em = rel_err(Ut[vs], Ur[vs]), rel_err(Um[vs], Ur[vs])
    print(f"{name}: FP32 tile {et:.2e}, FP32 march {em:.2e} (relative to the FP64 oracle)")
    assert em <= 1e-4
    assert em <= max(2.0 * et, 5e-6)      # both at FP32 rounding of a ~1e2 MPa state
    assert rel_err(Bm[:, g:-g], Br[:, g:-g]) <= 1e-3


WIDE_BOXES = [(0, 0, 299, 11), (0, 12, 130, 23), (131, 12, 299, 23)]


@pytest.mark.parametrize("name", ["rs_aging", "sw_ref9", "rs_free_edges"])
@pytest.mark.parametrize("boxes", [WIDE_BOXES, [(0, 0, 299, 23)]], ids=["three_patches", "one_patch"])
def test_wide_levels_match_oracle(cuda_lib, name, boxes):
    """A 300-column level: many marching strips side by side, strips that end
    short of a patch edge and fault-row strips finished after the fault kernel.
    FP64 form against the oracle at 1e-11; the mixed form against it at FP32
    rounding."""
    if name == "sw_ref9":
        sc = S.slip_weakening(nx=300, ny=24, dx=0.1, layout=A.TMK_SW_LAYOUT_REFERENCE9)
    else:
        sc = S.rate_state(nx=300, ny=24, dx=0.1)
    if name == "rs_free_edges":
        for k, v in enumerate((1, 1, 2, 1, 0, 0)):
            sc.scheme.boundary_type[k] = v
    sc.scheme.volume_kernel = A.TMK_VOLUME_MARCH
    rng = np.random.default_rng(7)
    U0 = perturbed_state(sc, rng, amp_v=0.05, amp_s=1.0)
    B0 = sc.initial_B()
    Ur, Br = U0.copy(), B0.copy()
    t = 0.0
    for _ in range(4):
        assert O.level_step(sc, Ur, Br, boxes, t, sc.dt()) == 0
        t += sc.dt()
    g = A.TMK_NGHOST
    vs = (slice(None), slice(g, -g), slice(g, -g))
    info64 = []
    Ug, Bg = _run_level(sc, boxes, U0, B0, 4, info64)
    assert rel_err(Ug[vs], Ur[vs]) <= 1e-11
    assert rel_err(Bg[:, g:-g], Br[:, g:-g]) <= 1e-11
    sc.scheme.precision = A.TMK_PREC_MIXED
    Um, Bm = _run_level(sc, boxes, U0, B0, 4)
    if name == "rs_free_edges":
        # Where the fault meets a free x edge, the FP64 form (the reference's
        # bracketed Newton iteration on the slip rate) ends friction solves of the
        # corner faces at the bracket or the iteration limit, while the mixed
        # form's solve (Newton on z = asinh(V / 2V0 e^(psi/a))) converges there: the
        # forms differ on those faces by design.  Away from the corners (13 cells:
        # the 4 steps' numerical domain of dependence, 3 cells a step) the mixed
        # form is FP32 rounding.
        assert info64[2] > 0, info64
        K = 13
        keep = np.ones(Ur.shape[1:], dtype=bool)
        keep[g:g + K, g:g + K] = False
        keep[g:g + K, -g - K:-g] = False
        keep = keep[g:-g, g:-g]
        assert rel_err(Um[vs][:, keep], Ur[vs][:, keep]) <= 1e-4
        return
    assert rel_err(Um[vs], Ur[vs]) <= 1e-4
    assert rel_err(Bm[:, g:-g], Br[:, g:-g]) <= 1e-3
