"""A rupture refined on the fly: three levels at ratio 4 over a slip-weakening
fault with Drucker-Prager plasticity (1 MPa cohesion, background normal
stresses from plas_Psi = 30 degrees), tagged on the fault row's slip rate and
on velocity gradients and regridded every 2 coarse steps (boxes of 8 to 64
cells from the tags) -- the 3-level AMR workload shrunk to a 64 x 32 base.

The device run (tags, prolongation, copy of the old levels, subcycled steps)
is compared with the oracle run given the same boxes: tags bit for bit; the
state and fault data of every level after each cycle of 2 coarse steps (32
finest substeps), and the new levels' prolonged and copied cells, to 1e-8
(FP64 form; the rounding differences grow with the rupture).  The regrid
sequence follows AMRLevelLinElast::regrid / AMR::regrid
(srcLinElast/AMRLevelLinElast.cpp:577-949): tag level l of the new hierarchy,
make the boxes of level l + 1, prolong them from level l, copy the cells the
old level l + 1 shares with them."""
import numpy as np
import pytest

import oracle as O
from tetemoko_gb300 import _capi as A, scenarios as S
from tests import amr_helpers as H

pytestmark = pytest.mark.gpu
G = A.TMK_NGHOST
RATIOS = [4, 4]
# FP64 device against FP64 oracle over a growing rupture: the rounding
# differences of the two builds are amplified by the rupture dynamics, by
# about tenfold per cycle (measured 1e-11 after the first cycle, 2.5e-10 after
# the second); a fault in a regrid operator shows at 1e-3 and above
RTOL_RUN = 1e-8
BOX_ARGS = dict(block_factor=8, max_grid_size=64, fill_ratio=0.7)


def _scenario():
    return S.slip_weakening(nx=64, ny=32, dx=0.1, plasticity=True, cohesion=1.0, plas_psi=30)


def _initial_levels(sc):
    Ug, Bg = sc.initial_U(), sc.initial_B()
    levels = [H.level_from_global((0, 0, sc.nx - 1, sc.ny - 1), sc.dx, H.L0_BOXES, sc.nbdry, Ug, Bg)]
    for boxes, r in zip(H.LAYOUTS[(4, 4)], RATIOS):
        c = levels[-1]
        f = O.LevelData(H.refine_domain(c.domain, r), c.dx / r, boxes, sc.nbdry)
        assert O.fine_interp(r, c, f) == 0
        levels.append(f)
    return levels


def _tag_params(level):
    return A.tag_params(level=level, refine_thresh=0.01, tag_buffer=2, slip_rate_thresh=1e-3)


def _copy_overlap(new: O.LevelData, old: O.LevelData):
    """The valid cells (and fault faces) new shares with old, copied from old."""
    for p, nb in enumerate(new.boxes):
        for q, ob in enumerate(old.boxes):
            x0, x1, y0, y1 = max(nb[0], ob[0]), min(nb[2], ob[2]), max(nb[1], ob[1]), min(nb[3], ob[3])
            if x0 > x1 or y0 > y1:
                continue
            dst = (slice(None), slice(y0 - nb[1] + G, y1 - nb[1] + G + 1), slice(x0 - nb[0] + G, x1 - nb[0] + G + 1))
            src = (slice(None), slice(y0 - ob[1] + G, y1 - ob[1] + G + 1), slice(x0 - ob[0] + G, x1 - ob[0] + G + 1))
            new.U[p][dst] = old.U[q][src]
            if new.B[p] is not None and old.B[q] is not None:
                new.B[p][:, x0 - nb[0] + G:x1 - nb[0] + G + 1] = old.B[q][:, x0 - ob[0] + G:x1 - ob[0] + G + 1]


def _worst(a: O.LevelData, b: O.LevelData):
    """(patch, state or fault component, relative error) of the largest difference."""
    from tests.helpers import rel_err
    out = (None, None, 0.0)
    for p in range(len(b.boxes)):
        for c in range(22):
            e = rel_err(a.U[p][c:c + 1, G:-G, G:-G], b.U[p][c:c + 1, G:-G, G:-G])
            if e > out[2]:
                out = (p, f"U{c}", e)
        if b.B[p] is not None:
            for c in range(b.B[p].shape[0]):
                e = rel_err(a.B[p][c:c + 1, G:-G], b.B[p][c:c + 1, G:-G])
                if e > out[2]:
                    out = (p, f"B{c}", e)
    return out


def test_regridded_ratio4_plastic_rupture_matches_oracle(cuda_lib):
    from tetemoko_gb300.amr import AMRHierarchy, regrid
    from tetemoko_gb300.level import Context
    from tests.test_gpu_amr import _levels_on_gpu, _read, _valid_err
    sc = _scenario()
    refs = _initial_levels(sc)
    ctx = Context(sc)
    lvs = _levels_on_gpu(ctx, refs)
    dt0 = sc.dt()
    t = 0.0
    sizes = set()
    for cycle in range(2):
        # two subcycled coarse steps on both sides
        h = AMRHierarchy(lvs, RATIOS, time=t)
        for _ in range(2):
            h.step(dt0)
        h.close()
        assert O.amr_run(sc, refs, RATIOS, t, dt0, 2) == 0
        t += 2 * dt0
        for l, (lv, r) in enumerate(zip(lvs, refs)):
            rc, info = lv.status()
            assert rc == 0, info
            got = _read(lv, r)
            err = _valid_err(got, r)
            print(f"cycle {cycle} level {l}: {err:.2e}")
            assert err <= RTOL_RUN, (cycle, l, _worst(got, r))
        # regrid on the device (tags, boxes, prolongation, copy of the old levels)
        old = lvs
        new = regrid(lvs, RATIOS, [_tag_params(0), _tag_params(1)], **BOX_ARGS)
        assert len(new) == 3, "both finer levels must be kept"
        # the oracle: the same tags from the same state, the same boxes, prolongation and copy
        new_refs = [refs[0]]
        for l in range(2):
            coarse = new_refs[l]
            want = O.tag_cells(sc, _tag_params(l), coarse.copy(), coarse=new_refs[l - 1] if l else None,
                               r=RATIOS[l - 1] if l else 2)
            got = new[l].tag_cells(_tag_params(l))
            np.testing.assert_array_equal(got, want)
            boxes = new[l + 1].boxes
            for b in boxes:
                sizes.add(max(b[2] - b[0] + 1, b[3] - b[1] + 1))
            fine = O.LevelData(H.refine_domain(coarse.domain, RATIOS[l]), coarse.dx / RATIOS[l], boxes, sc.nbdry)
            assert O.fine_interp(RATIOS[l], coarse, fine) == 0
            _copy_overlap(fine, refs[l + 1])
            new_refs.append(fine)
        for lv, d in zip(new[1:], new_refs[1:]):     # prolonged from levels that differ by rounding
            assert _valid_err(_read(lv, d), d) <= RTOL_RUN
        for lv in old[1:]:
            lv.close()
        lvs, refs = new, new_refs
    assert sizes and min(sizes) >= 8 and max(sizes) <= 64
    for lv in lvs:
        lv.close()
    ctx.close()
