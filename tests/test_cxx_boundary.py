"""The drop-in boundary compiled from C++: tests/cxx/chombo_shim.cpp holds the
bodies a Chombo build puts into LinElastPatchGodunov::updateState /
plasticUpdate and LinElastLevelGodunov::define / step
(srcLinElast/LinElastPatchGodunov.H:63-83, srcLinElast/LinElastLevelGodunov.H:91-114)
over stand-in Chombo classes.  It is compiled with g++ -Wall -Wextra -Werror
-pedantic against include/tetemoko_gb300.h and linked to the library, so a
struct-layout, const or signature mismatch a C++ caller would meet fails the
build.  Without a GPU the argument errors come back through MayDay; on the
GPU one patch step and several level steps through the shim equal the oracle."""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

import oracle as O
from tetemoko_gb300 import _capi as A, scenarios as S
from tests.helpers import RTOL_FP64, perturbed_state, rel_err

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cxx", "chombo_shim.cpp")
G = A.TMK_NGHOST


@pytest.fixture(scope="session")
def shim(cuda_lib, tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    libdir = os.path.dirname(A.lib_path())
    out = str(tmp_path_factory.mktemp("cxx") / "libchombo_shim.so")
    cmd = [cxx, "-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror", "-pedantic", "-fPIC", "-shared",
           "-I", os.path.join(ROOT, "include"), SRC, "-o", out,
           "-L", libdir, "-ltetemoko_gb300", f"-Wl,-rpath,{libdir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    lib = C.CDLL(out)
    vp, ip, dp, d = C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_double), C.c_double
    lib.shim_context_create.argtypes = [vp, vp, vp, vp, vp]
    lib.shim_patch_update_state.argtypes = [vp, ip, vp, ip, C.c_int, vp, vp, ip, ip, d, d, d, dp]
    lib.shim_plastic_update.argtypes = [vp, ip, ip, ip, d, d]
    lib.shim_level_define.argtypes = [ip, d, C.c_int, ip]
    lib.shim_level_set_patch.argtypes = [C.c_int, vp, vp, C.c_int]
    lib.shim_level_get_patch.argtypes = [C.c_int, vp, vp, C.c_int]
    lib.shim_level_step.argtypes = [d, d, dp]
    yield lib
    lib.shim_level_destroy()
    lib.shim_context_destroy()


def _iv(*v):
    return (C.c_int * len(v))(*v)


def _create(lib, sc):
    ref = lambda x: C.byref(x) if x is not None else None
    return lib.shim_context_create(C.byref(sc.elastic), C.byref(sc.scheme), ref(sc.rs), ref(sc.sw),
                                   ref(sc.plastic))


def test_shim_compiles_and_reports_argument_errors(shim):
    sc = S.rate_state(nx=32, ny=16)
    sc.scheme.use_char_limiting = 1                      # with primitive limiting: PPMNormalPred MayDay
    assert _create(shim, sc) == 5
    # no context: the ABI's BAD_DESC comes back through MayDay::Error
    U = np.zeros((22, 16 + 2 * G, 32 + 2 * G))
    mws = C.c_double()
    rc = shim.shim_patch_update_state(U.ctypes.data, _iv(-G, -G, 31 + G, 15 + G), None, None, 0, None, None,
                                      _iv(0, 0, 31, 15), _iv(0, 0, 31, 15), 0.1, 0.0, 0.01, C.byref(mws))
    assert rc == 1
    # a FluxBox whose face FABs do not cover the patch's faces (caught before the ABI)
    Fx = np.zeros((22, 16, 32))
    Fy = np.zeros((22, 17, 32))
    rc = shim.shim_patch_update_state(U.ctypes.data, _iv(-G, -G, 31 + G, 15 + G), None, None, 0, Fx.ctypes.data,
                                      Fy.ctypes.data, _iv(0, 0, 30, 15), _iv(0, 0, 31, 15), 0.1, 0.0, 0.01,
                                      C.byref(mws))
    assert rc == 1
    assert shim.shim_level_step(0.0, 0.01, C.byref(mws)) == 1   # no level defined


def test_shim_context_without_gpu_reports_no_device(shim):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    assert _create(shim, S.rate_state(nx=32, ny=16)) == 7


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["rs", "sw_plastic"])
def test_shim_patch_step_matches_oracle(shim, kind):
    import torch
    sc = S.rate_state(nx=64, ny=32, dx=0.1) if kind == "rs" else \
        S.slip_weakening(nx=64, ny=32, dx=0.1, plasticity=True)
    valid = (5, 0, 40, 13)
    rng = np.random.default_rng(77)
    ulo = (valid[0] - G, valid[1] - G)
    U0 = perturbed_state(sc, rng, lo=valid[:2], hi=valid[2:])
    nbx = valid[2] - valid[0] + 1 + 2 * G
    B0 = sc.initial_B(xlo=0, xhi=nbx - 1 - 2 * G)
    dt, time = sc.dt(), 0.75
    Ur, Br = U0.copy(), B0.copy()
    rc, Fxr, Fyr = O.patch_update_state(sc, Ur, ulo, valid[:2], valid[2:], Br, valid[0] - G, time, dt,
                                        with_flux=True)
    assert rc == 0
    if sc.plastic is not None:
        O.plastic_correction(sc, Ur, ulo, valid[:2], valid[2:], dt)
    assert _create(shim, sc) == 0
    Ud = torch.from_numpy(U0.copy()).cuda()
    Bd = torch.from_numpy(B0.copy()).cuda()
    nx, ny = valid[2] - valid[0] + 1, valid[3] - valid[1] + 1
    Fx = torch.empty((22, ny, nx + 1), dtype=torch.float64, device="cuda")
    Fy = torch.empty((22, ny + 1, nx), dtype=torch.float64, device="cuda")
    ubox = _iv(ulo[0], ulo[1], ulo[0] + U0.shape[2] - 1, ulo[1] + U0.shape[1] - 1)
    bbox = _iv(valid[0] - G, 0, valid[0] - G + nbx - 1, 0)
    mws = C.c_double()
    dom = _iv(0, 0, sc.nx - 1, sc.ny - 1)
    rc = shim.shim_patch_update_state(Ud.data_ptr(), ubox, Bd.data_ptr(), bbox, sc.nbdry, Fx.data_ptr(),
                                      Fy.data_ptr(), _iv(*valid), dom, sc.dx, time, dt, C.byref(mws))
    assert rc == 0
    if sc.plastic is not None:
        assert shim.shim_plastic_update(Ud.data_ptr(), ubox, _iv(*valid), dom, sc.dx, dt) == 0
    torch.cuda.synchronize()
    assert mws.value == max(sc.elastic.cs, sc.elastic.cp)
    vs = (slice(None), slice(G, -G), slice(G, -G))
    assert rel_err(Ud.cpu().numpy()[vs], Ur[vs]) <= RTOL_FP64
    ev = [c for c in range(22) if c % 11 < 9]
    assert rel_err(Fx.cpu().numpy()[ev], Fxr[ev]) <= RTOL_FP64
    assert rel_err(Fy.cpu().numpy()[ev], Fyr[ev]) <= RTOL_FP64
    assert rel_err(Bd.cpu().numpy()[:, G:-G], Br[:, G:-G]) <= RTOL_FP64
    shim.shim_context_destroy()


@pytest.mark.gpu
def test_shim_level_steps_match_oracle(shim):
    sc = S.rate_state(nx=64, ny=32, dx=0.1)
    boxes = [(0, 0, 20, 9), (21, 0, 63, 9), (0, 10, 31, 31), (32, 10, 47, 20), (32, 21, 47, 31), (48, 10, 63, 31)]
    rng = np.random.default_rng(78)
    Ug = perturbed_state(sc, rng, amp_v=0.05, amp_s=1.0)
    Bg = sc.initial_B()
    Ur, Br = Ug.copy(), Bg.copy()
    dt = sc.dt()
    for k in range(4):
        assert O.level_step(sc, Ur, Br, boxes, k * dt, dt) == 0
    assert _create(shim, sc) == 0
    flat = [v for b in boxes for v in b]
    assert shim.shim_level_define(_iv(0, 0, sc.nx - 1, sc.ny - 1), sc.dx, len(boxes), _iv(*flat)) == 0
    for p, b in enumerate(boxes):
        U = np.ascontiguousarray(Ug[:, b[1]:b[3] + 1 + 2 * G, b[0]:b[2] + 1 + 2 * G])
        B = np.ascontiguousarray(Bg[:, b[0]:b[2] + 1 + 2 * G]) if b[1] == 0 else None
        assert shim.shim_level_set_patch(p, U.ctypes.data, B.ctypes.data if B is not None else None, 1) == 0
    dtn = C.c_double()
    for k in range(4):
        assert shim.shim_level_step(k * dt, dt, C.byref(dtn)) == 0
    assert abs(dtn.value - sc.dx / max(sc.elastic.cs, sc.elastic.cp)) < 1e-15
    for p, b in enumerate(boxes):
        U = np.empty((22, b[3] - b[1] + 1 + 2 * G, b[2] - b[0] + 1 + 2 * G))
        B = np.empty((sc.nbdry, b[2] - b[0] + 1 + 2 * G)) if b[1] == 0 else None
        assert shim.shim_level_get_patch(p, U.ctypes.data, B.ctypes.data if B is not None else None, 1) == 0
        ys, xs = slice(b[1] + G, b[3] + 1 + G), slice(b[0] + G, b[2] + 1 + G)
        assert rel_err(U[:, G:-G, G:-G], Ur[:, ys, xs]) <= 1e-11
        if B is not None:
            assert rel_err(B[:, G:-G], Br[:, xs]) <= 1e-11
    shim.shim_level_destroy()
    shim.shim_context_destroy()
