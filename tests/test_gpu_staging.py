"""Setting and reading a level's state from pinned host memory (read and
written in place by the conversion kernels over the host link) gives the same
bits as from pageable memory (staged through a device buffer) and as from a
device tensor, in both forms."""
import numpy as np
import pytest

from tetemoko_gb300 import _capi as A, scenarios as S
from tests.helpers import perturbed_state

pytestmark = pytest.mark.gpu
BOXES = [(0, 0, 31, 15), (32, 0, 63, 15), (0, 16, 63, 31)]


@pytest.mark.parametrize("prec", [A.TMK_PREC_FP64, A.TMK_PREC_MIXED], ids=["fp64", "mixed"])
def test_pinned_pageable_and_device_buffers_agree(cuda_lib, prec):
    import torch
    from tetemoko_gb300.level import Context, LinElastLevelGodunov
    sc = S.rate_state(nx=64, ny=32, dx=0.1, precision=prec)
    Ug = perturbed_state(sc, np.random.default_rng(71), amp_v=0.05, amp_s=1.0)
    Bg = sc.initial_B()
    ctx = Context(sc)
    outs = []
    for mode in ("pageable", "pinned", "device"):
        lv = LinElastLevelGodunov(ctx, BOXES)   # a fresh level: the same buffer history in every mode
        lv.set_level(Ug, Bg)                    # known state, then overwritten patch by patch
        for p in range(len(BOXES)):
            U, B = lv.get_patch(p)
            if mode == "pinned":
                Ut = torch.from_numpy(U).pin_memory()
                Bt = torch.from_numpy(B).pin_memory() if B is not None else None
                lv.set_patch(p, Ut.numpy(), Bt.numpy() if Bt is not None else None)
            elif mode == "device":
                lv.set_patch(p, torch.from_numpy(U).cuda(), torch.from_numpy(B).cuda() if B is not None else None)
            else:
                lv.set_patch(p, U, B)
        for k in range(3):
            lv.step(k * sc.dt(), sc.dt())
        res = []
        for p in range(len(BOXES)):
            ushape, bshape = lv.patch_shapes(p)
            if mode == "pinned":
                Ut = torch.empty(ushape, dtype=torch.float64).pin_memory()
                Bt = torch.empty(bshape, dtype=torch.float64).pin_memory() if lv.touches_fault(p) else None
                lv.get_patch(p, Ut.numpy(), Bt.numpy() if Bt is not None else None)
                res.append((Ut.numpy().copy(), None if Bt is None else Bt.numpy().copy()))
            elif mode == "device":
                Ut = torch.empty(ushape, dtype=torch.float64, device="cuda")
                Bt = torch.empty(bshape, dtype=torch.float64, device="cuda") if lv.touches_fault(p) else None
                lv.get_patch(p, Ut, Bt)
                res.append((Ut.cpu().numpy(), None if Bt is None else Bt.cpu().numpy()))
            else:
                res.append(lv.get_patch(p))
        outs.append(res)
        lv.close()
    for other in outs[1:]:
        for (ua, ba), (ub, bb) in zip(outs[0], other):
            np.testing.assert_array_equal(ua, ub)
            if ba is not None:
                np.testing.assert_array_equal(ba, bb)
    ctx.close()
