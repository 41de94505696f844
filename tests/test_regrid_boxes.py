"""Host box generation of a regrid (Berger-Rigoutsos clustering over the tags,
blocking factor, maximum box size, proper nesting): properties on CPU."""
import numpy as np

from tetemoko_gb300.amr import boxes_from_tags


def _cells(boxes, r):
    s = set()
    for b in boxes:
        for j in range(b[1] // r, b[3] // r + 1):
            for i in range(b[0] // r, b[2] // r + 1):
                s.add((i, j))
    return s


def _allowed_block(i, j, domain, nest, buf, b):
    """The tag's b x b block lies in the nesting boxes' union shrunk by buf
    cells (not against the domain's edges)."""
    x0, y0 = (i - domain[0]) // b * b + domain[0], (j - domain[1]) // b * b + domain[1]
    for y in range(y0, y0 + b):
        for x in range(x0, x0 + b):
            for dy in range(-buf, buf + 1):
                for dx in range(-buf, buf + 1):
                    xx = min(max(x + dx, domain[0]), domain[2])
                    yy = min(max(y + dy, domain[1]), domain[3])
                    if not any(n[0] <= xx <= n[2] and n[1] <= yy <= n[3] for n in nest):
                        return False
    return True


def _check(mask, domain, r, bf, maxg, boxes, nest=None, buf=1):
    fine = [(domain[0] * r, domain[1] * r, (domain[2] + 1) * r - 1, (domain[3] + 1) * r - 1)]
    for b in boxes:
        assert b[0] >= fine[0][0] and b[1] >= fine[0][1] and b[2] <= fine[0][2] and b[3] <= fine[0][3]
        for k in range(2):
            assert b[k] % bf == 0 and (b[k + 2] + 1) % bf == 0          # blocking factor
            assert b[k + 2] - b[k] + 1 <= maxg                           # maximum box size
    for a in range(len(boxes)):                                          # disjoint
        for c in range(a):
            p, q = boxes[a], boxes[c]
            assert p[2] < q[0] or q[2] < p[0] or p[3] < q[1] or q[3] < p[1]
    covered = _cells(boxes, r)
    ys, xs = np.nonzero(mask)
    for i, j in zip(xs + domain[0], ys + domain[1]):
        inside = nest is None or _allowed_block(i, j, domain, nest, buf, max(1, bf // r))
        if inside:
            assert (i, j) in covered                                     # every nested tag refined
    if nest is not None:                                                 # proper nesting
        for i, j in covered:
            assert any(n[0] <= i <= n[2] and n[1] <= j <= n[3] for n in nest)


def test_two_clusters_give_two_boxes():
    mask = np.zeros((64, 128), dtype=np.uint8)
    mask[0:6, 10:30] = 1
    mask[20:40, 90:100] = 1
    boxes = boxes_from_tags(mask, (0, 0, 127, 63), ratio=2, block_factor=8, max_grid_size=128)
    _check(mask, (0, 0, 127, 63), 2, 8, 128, boxes)
    assert len(boxes) == 2


def test_random_tags_respect_every_constraint():
    rng = np.random.default_rng(5)
    for trial in range(8):
        mask = (rng.random((96, 160)) < 0.03).astype(np.uint8)
        mask[40:60, 50:110] = 1
        for r, bf, maxg in ((2, 8, 64), (4, 16, 128), (2, 4, 32)):
            boxes = boxes_from_tags(mask, (0, 0, 159, 95), ratio=r, block_factor=bf, max_grid_size=maxg,
                                    fill_ratio=0.7)
            _check(mask, (0, 0, 159, 95), r, bf, maxg, boxes)


def test_boxes_nest_in_the_coarser_level():
    mask = np.zeros((64, 128), dtype=np.uint8)
    mask[5:30, 20:100] = 1
    nest = [(0, 0, 63, 31), (64, 0, 95, 31)]       # the level's patches: x beyond 95 is not covered
    boxes = boxes_from_tags(mask, (0, 0, 127, 63), ratio=2, block_factor=4, max_grid_size=64,
                            nest_boxes=nest, nest_buffer=1)
    _check(mask, (0, 0, 127, 63), 2, 4, 64, boxes, nest=nest, buf=1)
    assert boxes
