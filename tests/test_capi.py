"""The C-ABI library without a GPU: it loads, exports every declared entry
point, and rejects bad arguments with the documented status codes before it
touches a device."""
import ctypes as C
import os
import re

import pytest

from tetemoko_gb300 import _capi as A, scenarios as S

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include",
                      "tetemoko_gb300.h")


def declared_functions():
    with open(HEADER) as f:
        src = f.read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(tmk_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_the_drop_in_entry_points():
    names = declared_functions()
    for n in ("tmk_context_create", "tmk_patch_update_state", "tmk_plastic_update", "tmk_level_create",
              "tmk_level_step", "tmk_level_status", "tmk_max_wave_speed"):
        assert n in names


def test_library_exports_every_declared_symbol(cuda_lib):
    missing = [n for n in declared_functions() if not hasattr(cuda_lib, n)]
    assert not missing, missing


def test_abi_version(cuda_lib):
    assert cuda_lib.tmk_abi_version() == 5


def _create(lib, sc, rs=True, sw=False, pl=False):
    h = C.c_void_p()
    rc = lib.tmk_context_create(C.byref(sc.elastic), C.byref(sc.scheme),
                                C.byref(sc.rs) if (rs and sc.rs is not None) else None,
                                C.byref(sc.sw) if (sw and sc.sw is not None) else None,
                                C.byref(sc.plastic) if (pl and sc.plastic is not None) else None, C.byref(h))
    return rc, h


def test_context_argument_errors(cuda_lib):
    lib = cuda_lib
    sc = S.rate_state(nx=32, ny=16)
    assert lib.tmk_context_create(None, None, None, None, None, None) == 1          # TMK_ERR_BAD_DESC
    h = C.c_void_p()
    assert lib.tmk_context_create(None, C.byref(sc.scheme), None, None, None, C.byref(h)) == 1
    # the rate-and-state plug-in needs its parameters
    rc, _ = _create(lib, sc, rs=False)
    assert rc == 1
    # limiting in primitive AND characteristic variables: PPMNormalPred MayDay -> unsupported
    sc2 = S.rate_state(nx=32, ny=16)
    sc2.scheme.use_char_limiting = 1
    assert _create(lib, sc2)[0] == 5
    # a normal predictor order other than CTU (0), PLM (1), PPM (2)
    sc3 = S.rate_state(nx=32, ny=16)
    sc3.scheme.normal_pred_order = 3
    assert _create(lib, sc3)[0] == 5
    # invalid boundary type ("Invalid Boundary Type")
    sc4 = S.rate_state(nx=32, ny=16)
    sc4.scheme.boundary_type[1] = 7
    assert _create(lib, sc4)[0] == 1
    # cp < cs breaks the characteristic ordering the transforms assume
    sc5 = S.rate_state(nx=32, ny=16)
    sc5.elastic.cp = 1.0
    assert _create(lib, sc5)[0] == 1


def test_context_without_gpu_reports_no_device(cuda_lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    rc, h = _create(cuda_lib, S.rate_state(nx=32, ny=16))
    assert rc == 7                                                                     # TMK_ERR_NO_DEVICE
    assert not h.value


def test_null_handles_are_rejected(cuda_lib):
    lib = cuda_lib
    assert lib.tmk_level_step(None, 0.0, 0.1, None, None) == 1
    assert lib.tmk_patch_update_state(None, None, None, None, None, None, None, 0.1, 0.0, 0.1, None, None) == 1
    assert lib.tmk_patch_update_state_noalloc(None, None, None, None, None, None, None, 0.1, 0.0, 0.1, None,
                                              None) == 1
    out = (C.c_double * 5)()
    assert lib.tmk_context_constants(None, out) == 1
    # the 3-D level: no context, no handle
    dom = A.box3((0, 0, 0), (7, 7, 7))
    boxes = (A.Box3 * 1)(A.box3((0, 0, 0), (7, 7, 7)))
    h = C.c_void_p()
    assert lib.tmk_level3d_create(None, C.byref(dom), 0.1, 1, boxes, C.byref(h)) == 1
    assert not h.value
    assert lib.tmk_level3d_step(None, 0.0, 0.1, None, None) == 1
    assert lib.tmk_level3d_exchange(None, None) == 1
    assert lib.tmk_level3d_set_patch(None, 0, None, None, 1) == 1
    assert lib.tmk_level3d_get_patch(None, 0, None, None, 1) == 1
    assert lib.tmk_level3d_patch_fabs(None, 0, None, None) == 1
    lib.tmk_context_destroy(None)
    lib.tmk_level_destroy(None)
    lib.tmk_level3d_destroy(None)
