"""Shared builders of the AMR tests: seeded level states and hierarchy layouts."""
from __future__ import annotations

import numpy as np

import oracle as O
from tetemoko_gb300 import _capi as A
from tests.helpers import perturbed_state

G = A.TMK_NGHOST

# level 0: 64 x 32 cells of 0.1 km in six patches; level 1 (ratio 2) around the
# nucleation at x = 3.2 km on the fault; level 2 (ratio 2) inside level 1
L0_BOXES = [(0, 0, 20, 9), (21, 0, 63, 9), (0, 10, 31, 31), (32, 10, 47, 20), (32, 21, 47, 31), (48, 10, 63, 31)]
L1_BOXES = [(40, 0, 71, 15), (72, 0, 87, 23), (40, 16, 71, 23)]
L2_BOXES = [(96, 0, 127, 31), (128, 0, 143, 31)]

# the reference decks' refinement ratios (4: execLinElast/tpv5_r1:69,
# input/bssa_flat_amr.input:84; 8: input/labvalues_Psi50_m.input:78): finer
# boxes of uneven size (8 to 64 cells per side) around the same nucleation,
# aligned to the ratio and nested at least 8 coarser cells inside their level
LAYOUTS = {
    (2, 2): [L1_BOXES, L2_BOXES],
    (4, 4): [[(96, 0, 159, 31), (160, 0, 167, 47), (168, 0, 175, 47), (96, 32, 159, 47)],
             [(448, 0, 575, 63), (576, 0, 639, 31)]],
    (4, 2): [[(96, 0, 159, 31), (160, 0, 167, 47), (168, 0, 175, 47), (96, 32, 159, 47)],
             [(224, 0, 287, 15), (288, 0, 319, 31)]],
    (8,): [[(192, 0, 319, 63), (320, 0, 351, 31)]],
}


def level_from_global(domain, dx, boxes, nb, Ug, Bg) -> O.LevelData:
    """Per-patch arrays sliced from a domain-wide state (22, ny+8, nx+8) and fault row (nb, nx+8)."""
    U, B = [], []
    for b in boxes:
        ys = slice(b[1] - domain[1], b[3] - domain[1] + 1 + 2 * G)
        xs = slice(b[0] - domain[0], b[2] - domain[0] + 1 + 2 * G)
        U.append(np.ascontiguousarray(Ug[:, ys, xs]))
        B.append(np.ascontiguousarray(Bg[:, xs]) if (nb > 0 and b[1] == domain[1]) else None)
    return O.LevelData(domain, dx, boxes, nb, U, B)


def refine_domain(d, r):
    return (d[0] * r, d[1] * r, (d[2] + 1) * r - 1, (d[3] + 1) * r - 1)


def hierarchy(sc, rng, nlev=2, ratios=(2, 2), fine_noise=0.0):
    """Level data of a hierarchy: level 0 seeded, finer levels prolonged from
    their coarser level (plus optional seeded noise).  The finer levels' boxes
    are LAYOUTS[ratios]."""
    nb = sc.nbdry
    dom0 = (0, 0, sc.nx - 1, sc.ny - 1)
    Ug = perturbed_state(sc, rng, amp_v=0.05, amp_s=1.0)
    Bg = sc.initial_B() if nb else np.zeros((0, sc.nx + 2 * G))
    levels = [level_from_global(dom0, sc.dx, L0_BOXES, nb, Ug, Bg)]
    boxes = LAYOUTS[tuple(ratios)]
    for l in range(1, nlev):
        r = ratios[l - 1]
        c = levels[-1]
        dom = refine_domain(c.domain, r)
        f = O.LevelData(dom, c.dx / r, boxes[l - 1], nb)
        assert O.fine_interp(r, c, f) == 0
        if fine_noise:
            for u in f.U:
                u[:3] += fine_noise * rng.standard_normal(u[:3].shape)
        levels.append(f)
    return levels


def composite_sum(levels, ratios):
    """Sum over the composite grid (cells not covered by a finer level) of U * cell area."""
    tot = np.zeros(22)
    for l, lv in enumerate(levels):
        covered = []
        if l + 1 < len(levels):
            r = ratios[l]
            covered = [(b[0] // r, b[1] // r, b[2] // r, b[3] // r) for b in levels[l + 1].boxes]
        for p, b in enumerate(lv.boxes):
            u = lv.U[p][:, G:-G, G:-G]
            yy, xx = np.mgrid[b[1]:b[3] + 1, b[0]:b[2] + 1]
            m = np.ones(xx.shape, bool)
            for c in covered:
                m &= ~((xx >= c[0]) & (xx <= c[2]) & (yy >= c[1]) & (yy <= c[3]))
            tot += (u * m).sum(axis=(1, 2)) * lv.dx ** 2
    return tot
