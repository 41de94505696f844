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
