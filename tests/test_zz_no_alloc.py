"""The allocation-free patch step gives the same answer as the allocating one.

tmk_patch_update_state_noalloc serves callers that cannot allocate device
memory while they step (their memory pool already owns the GPU, or they cannot
take cudaMalloc's device-wide synchronisation mid-step); its temporaries live
in a fixed device array shared by all calls.  This file is collected last so a
run that stops at the first failure has already run every other test; it also
passes on its own in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

from tetemoko_gb300 import _capi as A, scenarios as S
from tests.helpers import RTOL_FP64, perturbed_state, rel_err

pytestmark = pytest.mark.gpu


def _fab(t, lo0, lo1):
    f = A.Fab()
    f.data = t.data_ptr()
    f.lo[0], f.lo[1] = lo0, lo1
    f.hi[0], f.hi[1] = lo0 + t.shape[-1] - 1, lo1 + t.shape[-2] - 1
    f.ncomp = t.shape[0]
    return f


def _bfab(t, lo0, j0):
    f = A.Fab()
    f.data = t.data_ptr()
    f.lo[0], f.lo[1] = lo0, j0
    f.hi[0], f.hi[1] = lo0 + t.shape[-1] - 1, j0
    f.ncomp = t.shape[0]
    return f


def _step(lib, fn, ctx, U, ulo, B, bxlo, valid, domain, dx, time, dt, with_flux=True):
    import torch
    nx, ny = valid[2] - valid[0] + 1, valid[3] - valid[1] + 1
    Fx = Fy = None
    if with_flux:
        Fx = torch.empty((22, ny, nx + 1), dtype=torch.float64, device="cuda")
        Fy = torch.empty((22, ny + 1, nx), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    mws = C.c_double(0.0)
    rc = getattr(lib, fn)(ctx, C.byref(_fab(U, *ulo)), C.byref(_bfab(B, bxlo, domain[1])) if B is not None else None,
                          C.byref(_fab(Fx, valid[0], valid[1])) if with_flux else None,
                          C.byref(_fab(Fy, valid[0], valid[1])) if with_flux else None,
                          C.byref(A.box(*valid)), C.byref(A.box(*domain)), dx, time, dt, C.byref(mws), None)
    torch.cuda.synchronize()
    return rc, Fx, Fy, mws.value, free0 - torch.cuda.mem_get_info()[0]


# (valid box, fault data given, fluxes requested): a fault patch with fluxes;
# an interior patch without fault data; a fault patch without fluxes; a patch
# whose tile list needs more than one block of the set-up kernel (>256 tiles of
# 16 x 8) that still fits in the scratch
CASES = [((8, 0, 71, 29), True, True), ((20, 12, 83, 45), False, True), ((8, 0, 71, 29), True, False),
         ((4, 0, 203, 171), True, True)]


@pytest.mark.parametrize("valid,with_B,with_flux", CASES, ids=["fault_flux", "interior", "no_flux", "many_tiles"])
def test_noalloc_matches_allocating_entry_point_twice(cuda_lib, valid, with_B, with_flux):
    import torch
    from tetemoko_gb300.level import Context
    sc = S.rate_state(nx=224, ny=176, dx=0.1)
    ctx = Context(sc)
    lib = cuda_lib
    g = A.TMK_NGHOST
    domain = (0, 0, sc.nx - 1, sc.ny - 1)
    ulo = (valid[0] - g, valid[1] - g)
    bxlo = valid[0] - g
    rng = np.random.default_rng(2024)
    U0 = perturbed_state(sc, rng, lo=valid[:2], hi=valid[2:], amp_v=0.2, amp_s=2.0)
    B0 = sc.initial_B(xlo=valid[0], xhi=valid[2]) if with_B else None
    Ua, Ub = torch.from_numpy(U0.copy()).cuda(), torch.from_numpy(U0.copy()).cuda()
    Ba = torch.from_numpy(B0.copy()).cuda() if with_B else None
    Bb = torch.from_numpy(B0.copy()).cuda() if with_B else None
    dt = sc.dt()
    t = 0.5
    for call in range(2):
        ra, Fxa, Fya, ma, _ = _step(lib, "tmk_patch_update_state", ctx.h, Ua, ulo, Ba, bxlo, valid, domain, sc.dx,
                                    t, dt, with_flux)
        rb, Fxb, Fyb, mb, used = _step(lib, "tmk_patch_update_state_noalloc", ctx.h, Ub, ulo, Bb, bxlo, valid,
                                       domain, sc.dx, t, dt, with_flux)
        assert ra == A.TMK_OK and rb == A.TMK_OK, (call, ra, rb)
        assert ma == mb
        if call > 0:              # after the first call's set-up: no device memory taken
            assert used == 0, used
        assert rel_err(Ub.cpu().numpy(), Ua.cpu().numpy()) <= RTOL_FP64, call
        if with_B:
            assert rel_err(Bb.cpu().numpy(), Ba.cpu().numpy()) <= RTOL_FP64, call
        if with_flux:
            assert rel_err(Fxb.cpu().numpy(), Fxa.cpu().numpy()) <= RTOL_FP64, call
            assert rel_err(Fyb.cpu().numpy(), Fya.cpu().numpy()) <= RTOL_FP64, call
        # the step changed the state (a second call starts from new data)
        assert not np.array_equal(Ua.cpu().numpy(), U0)
        t += dt
    ctx.close()


def test_noalloc_refuses_a_patch_larger_than_its_scratch(cuda_lib):
    import torch
    from tetemoko_gb300.level import Context
    sc = S.rate_state(nx=512, ny=256, dx=0.1)
    ctx = Context(sc)
    g = A.TMK_NGHOST
    valid = (0, 0, 511, 255)   # the 520 x 264 x 22 updated state alone exceeds the fixed scratch
    assert 22 * 8 * (512 + 2 * g) * (256 + 2 * g) > A.TMK_NOALLOC_SCRATCH_BYTES
    U = torch.zeros((22, 256 + 2 * g, 512 + 2 * g), dtype=torch.float64, device="cuda")
    B = torch.zeros((A.TMK_RS_NBDRY, 512 + 2 * g), dtype=torch.float64, device="cuda")
    rc, *_ = _step(cuda_lib, "tmk_patch_update_state_noalloc", ctx.h, U, (-g, -g), B, -g, valid,
                   (0, 0, sc.nx - 1, sc.ny - 1), sc.dx, 0.0, sc.dt())
    assert rc == A.TMK_ERR_TOO_LARGE
    ctx.close()
