"""Checkpoint and restart: a subcycled hierarchy (with per-face friction on its
levels) saved between coarse steps and reloaded into new contexts and levels
continues bit for bit."""
import numpy as np
import pytest

from tetemoko_gb300 import _capi as A, scenarios as S
from tests import amr_helpers as H

pytestmark = pytest.mark.gpu
G = A.TMK_NGHOST


@pytest.mark.parametrize("prec", [A.TMK_PREC_FP64, A.TMK_PREC_MIXED], ids=["fp64", "mixed"])
def test_restart_continues_bit_for_bit(cuda_lib, prec, tmp_path):
    from tetemoko_gb300 import checkpoint
    from tetemoko_gb300.amr import AMRHierarchy
    from tetemoko_gb300.level import Context
    from tests.test_gpu_amr import _levels_on_gpu
    sc = S.rate_state(nx=64, ny=32, dx=0.1, precision=prec, plasticity=True)
    datas = H.hierarchy(sc, np.random.default_rng(101), nlev=3)
    ctx = Context(sc)
    lvs = _levels_on_gpu(ctx, datas)
    for l, lv in enumerate(lvs):
        lv.set_level_friction(S.friction_field(sc, refine=2 ** l))
    h = AMRHierarchy(lvs, [2, 2])
    dt = sc.dt()
    for _ in range(2):
        h.step(dt)
    path = str(tmp_path / "ckpt.npz")
    checkpoint.save(path, sc, lvs, [2, 2], h.time(0))
    for _ in range(2):
        h.step(dt)
    ref = [lv.get_patches() for lv in lvs]
    sc2, ctx2, lvs2, ratios, t = checkpoint.load(path)
    assert ratios == [2, 2] and abs(t - 2 * dt) < 1e-15
    h2 = AMRHierarchy(lvs2, ratios, time=t)
    for _ in range(2):
        h2.step(dt)
    for (Ua, Ba), lv in zip(ref, lvs2):
        Ub, Bb = lv.get_patches()
        for p in range(len(Ua)):
            np.testing.assert_array_equal(Ub[p][:, G:-G, G:-G], Ua[p][:, G:-G, G:-G])
            if Ba[p] is not None:
                np.testing.assert_array_equal(Bb[p][:, G:-G], Ba[p][:, G:-G])
    h.close(); h2.close()
    for lv in lvs + lvs2:
        lv.close()
    ctx.close(); ctx2.close()


@pytest.mark.parametrize("prec", [A.TMK_PREC_FP64, A.TMK_PREC_MIXED], ids=["fp64", "mixed"])
def test_3d_level_restart_continues_bit_for_bit(cuda_lib, prec, tmp_path):
    """A rate-and-state 3-D level on uneven patches, saved after two steps and
    reloaded into a new context and level, takes the same next two steps."""
    from tetemoko_gb300 import checkpoint
    from tetemoko_gb300.level import Context, LinElastLevelGodunov3D
    from tests.helpers import perturbed_state_3d, random_B_3d
    from tests.test_gpu_3d import DOM, LEVEL_TILINGS, NX, NY, NZ
    sc = S.rate_state(nx=NX, ny=NY, dx=0.1, precision=prec)
    rng = np.random.default_rng(202)
    U0 = perturbed_state_3d(sc, rng, DOM[0], DOM[1])
    B0 = random_B_3d(sc, rng, NX + 2 * G, NZ + 2 * G)
    tiles = LEVEL_TILINGS["uneven"]
    ctx = Context(sc)
    lvl = LinElastLevelGodunov3D(ctx, tiles, DOM)
    for p, ((l0, l1, l2), (h0, h1, h2)) in enumerate(tiles):
        U = np.ascontiguousarray(U0[:, l2:h2 + 2 * G + 1, l1:h1 + 2 * G + 1, l0:h0 + 2 * G + 1])
        B = np.ascontiguousarray(B0[:, l2:h2 + 2 * G + 1, l0:h0 + 2 * G + 1]) if lvl.touches_fault(p) else None
        lvl.set_patch(p, U, B)
    dt = sc.dt() / 3 ** 0.5
    for k in range(2):
        lvl.step(k * dt, dt)
    path = str(tmp_path / "ckpt3d.npz")
    checkpoint.save_3d(path, sc, lvl, 2 * dt)
    for k in range(2, 4):
        lvl.step(k * dt, dt)
    ref = [lvl.get_patch(p) for p in range(len(tiles))]
    sc2, ctx2, lvl2, t = checkpoint.load_3d(path)
    assert abs(t - 2 * dt) < 1e-15 and lvl2.boxes == lvl.boxes
    for k in range(2):
        lvl2.step(t + k * dt, dt)
    for p, (Ua, Ba) in enumerate(ref):
        Ub, Bb = lvl2.get_patch(p)
        np.testing.assert_array_equal(Ub[:, G:-G, G:-G, G:-G], Ua[:, G:-G, G:-G, G:-G])
        if Ba is not None:
            np.testing.assert_array_equal(Bb[:, G:-G, G:-G], Ba[:, G:-G, G:-G])
    lvl.close(); lvl2.close()
    ctx.close(); ctx2.close()
