"""A whole regrid cycle without Chombo: tags on the device, boxes on the host
(amr.boxes_from_tags), the new fine level prolonged and given the old fine
level's overlapping cells, then subcycled steps on the new hierarchy."""
import numpy as np
import pytest

from tetemoko_gb300 import _capi as A, scenarios as S
from tests import amr_helpers as H

pytestmark = pytest.mark.gpu
G = A.TMK_NGHOST


@pytest.mark.parametrize("r", [2, 4])
def test_regrid_cycle(cuda_lib, r):
    from tetemoko_gb300.amr import AMRHierarchy, regrid
    from tetemoko_gb300.level import Context
    from tests.test_gpu_amr import _levels_on_gpu
    sc = S.rate_state(nx=64, ny=32, dx=0.1)
    datas = H.hierarchy(sc, np.random.default_rng(91), nlev=2, ratios=(r, r))
    ctx = Context(sc)
    lvs = _levels_on_gpu(ctx, datas)
    h = AMRHierarchy(lvs, [r])
    for _ in range(2):
        h.step(sc.dt())
    t = h.time(0)
    h.close()
    tp = A.tag_params(level=0, refine_thresh=0.02, tag_buffer=1)
    mask = lvs[0].tag_cells(tp)
    old = {p: u for p, u in enumerate(lvs[1].get_patches()[0])}
    new = regrid(lvs, [r], [tp], block_factor=8, max_grid_size=32, fill_ratio=0.7)
    assert len(new) == 2 and new[0] is lvs[0]
    fine = new[1]
    # every tag is refined (level 0 nests everything), boxes obey the limits
    ys, xs = np.nonzero(mask)
    for i, j in zip(xs, ys):
        assert any(b[0] <= r * i <= b[2] and b[1] <= r * j <= b[3] for b in fine.boxes)
    for b in fine.boxes:
        assert b[2] - b[0] + 1 <= 32 and b[3] - b[1] + 1 <= 32 and b[0] % 8 == 0 and b[1] % 8 == 0
    # cells the old fine level had keep their values
    Un, _ = fine.get_patches()
    ob = lvs[1].boxes
    checked = 0
    for p, b in enumerate(fine.boxes):
        for q, c in enumerate(ob):
            x0, y0, x1, y1 = max(b[0], c[0]), max(b[1], c[1]), min(b[2], c[2]), min(b[3], c[3])
            if x0 > x1 or y0 > y1:
                continue
            a = Un[p][:, y0 - b[1] + G:y1 - b[1] + G + 1, x0 - b[0] + G:x1 - b[0] + G + 1]
            o = old[q][:, y0 - c[1] + G:y1 - c[1] + G + 1, x0 - c[0] + G:x1 - c[0] + G + 1]
            np.testing.assert_array_equal(a, o)
            checked += a.size
    assert checked > 0
    lvs[1].close()
    h2 = AMRHierarchy(new, [r], time=t)
    for _ in range(2):
        h2.step(sc.dt())
    for lv in new:
        assert lv.status()[0] == 0
        U, _ = lv.get_patches()
        assert all(np.isfinite(u[:, G:-G, G:-G]).all() for u in U)
    h2.close()
    for lv in new:
        lv.close()
    ctx.close()
