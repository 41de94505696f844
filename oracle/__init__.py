"""CPU FP64 oracle of tetemoko's per-level Godunov step -- TEST INFRASTRUCTURE.

Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline use this
package, and only as the checker: the CUDA product never imports or calls it.
The C++ source (tmk_oracle.cpp) restates the reference's Fortran kernels and
patch/level call order; its header lists the files it follows.

Parity status: the reference kernels themselves (srcLinElast/*.ChF,
ibcLinElast/*.ChF) cannot be compiled here (no Fortran compiler, no Chombo),
and the reference ships no tests or golden vectors, so parity with the
reference is unpinned.  The restatement is pinned instead by known-answer
properties of the reference formulas (tests/test_oracle_kat.py) and by exact
solutions of the equations it discretises (tests/test_oracle_waves.py: plane
waves in 2-D and 3-D, also through a refined hierarchy and at free and
absorbing edges, converging at the scheme's order; uniformly sliding
slip-weakening and rate-and-state faults meeting their 1-D answers; a uniform
over-stressed state relaxing by the closed form of the plastic return).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from tetemoko_gb300 import _capi as A

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "tmk_oracle.cpp")
LIB = os.path.join(HERE, "libtmk_oracle.so")

_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle with g++ (-O2, no FMA contraction, OpenMP)."""
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fopenmp", "-shared", "-fPIC",
               "-o", LIB + ".tmp", SRC]
        subprocess.run(cmd, check=True)
        os.replace(LIB + ".tmp", LIB)
    return LIB


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        P = C.POINTER
        dp, ip = P(C.c_double), P(C.c_int)
        E, S, R, W, PL = (P(A.ElasticParams), P(A.Scheme), P(A.RSParams), P(A.SWParams),
                          P(A.PlasticParams))
        L.tmko_constants.argtypes = [E, dp]
        L.tmko_charanalysis.argtypes = [E, dp, C.c_int]
        L.tmko_charsynthesis.argtypes = [E, dp, C.c_int]
        L.tmko_riemann.argtypes = [E, dp, dp, dp, C.c_int]
        L.tmko_edgebc.argtypes = [E, dp, dp, C.c_int, C.c_int, C.c_int]
        L.tmko_rsnewton.argtypes = [E, R, C.c_double, C.c_double, C.c_double, C.c_double, dp, dp]
        L.tmko_rsfault.argtypes = [E, R, dp, dp, C.c_double, C.c_double]
        L.tmko_swfault.argtypes = [E, W, dp, dp, dp, C.c_double]
        L.tmko_plasticflow.argtypes = [E, PL, dp, C.c_double]
        L.tmko_patch_update_state.argtypes = [E, S, R, W, dp, ip, ip, dp, C.c_int, C.c_int, dp, dp,
                                              ip, ip, ip, ip, C.c_double, C.c_double, C.c_double]
        L.tmko_plastic_correction.argtypes = [E, PL, dp, ip, ip, ip, ip, C.c_double]
        L.tmko_patch_update_state_3d.argtypes = [E, S, R, W, dp, ip, ip, dp, ip, ip, dp, dp, dp,
                                                 ip, ip, ip, ip, C.c_double, C.c_double, C.c_double]
        L.tmko_plastic_correction_3d.argtypes = [E, PL, dp, ip, ip, ip, ip, C.c_double]
        L.tmko_level_step.argtypes = [E, S, R, W, PL, ip, ip, C.c_int, ip, dp, dp, C.c_double,
                                      C.c_double, C.c_double, C.c_int]
        L.tmko_level_step_fric.argtypes = [E, S, R, W, PL, ip, ip, C.c_int, ip, dp, dp, dp, C.c_double,
                                           C.c_double, C.c_double, C.c_int]
        LV = P(_Level)
        L.tmko_cf_fill.argtypes = [C.c_int, C.c_int, LV, LV, C.c_double, LV]
        L.tmko_average_down.argtypes = [C.c_int, C.c_int, LV, LV]
        L.tmko_fine_interp.argtypes = [C.c_int, C.c_int, LV, LV]
        L.tmko_register_entries.argtypes = [C.c_int, LV, LV, ip]
        L.tmko_tag_cells.argtypes = [E, S, R, W, P(A.TagParams), C.c_int, LV, LV, C.c_void_p]
        L.tmko_amr_run.argtypes = [E, S, R, W, PL, C.c_int, LV, ip, C.c_double, C.c_double, C.c_int, C.c_int]
        _lib = L
    return _lib


class _Level(C.Structure):
    _fields_ = [("dom", C.c_int * 4), ("dx", C.c_double), ("npatch", C.c_int),
                ("boxes", C.POINTER(C.c_int)), ("U", C.POINTER(C.c_double)), ("B", C.POINTER(C.c_double))]


def _dp(a: np.ndarray | None):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _iv(*v):
    return (C.c_int * len(v))(*v)


def _ref(x):
    return C.byref(x) if x is not None else None


# ------------------------------------------------------------- pointwise --
def constants(sc) -> dict:
    out = np.zeros(5)
    lib().tmko_constants(C.byref(sc.elastic), _dp(out))
    return dict(rho=out[0], lam=out[1], K=out[2], Zs=out[3], Zp=out[4])


def charanalysis(sc, w: np.ndarray, idir: int) -> np.ndarray:
    w = np.ascontiguousarray(w, dtype=np.float64).copy()
    lib().tmko_charanalysis(C.byref(sc.elastic), _dp(w), idir)
    return w


def charsynthesis(sc, w: np.ndarray, idir: int) -> np.ndarray:
    w = np.ascontiguousarray(w, dtype=np.float64).copy()
    lib().tmko_charsynthesis(C.byref(sc.elastic), _dp(w), idir)
    return w


def riemann(sc, wl, wr, idir: int) -> np.ndarray:
    g = np.zeros(22)
    wl = np.ascontiguousarray(wl, dtype=np.float64)
    wr = np.ascontiguousarray(wr, dtype=np.float64)
    lib().tmko_riemann(C.byref(sc.elastic), _dp(g), _dp(wl), _dp(wr), idir)
    return g


def edge_bc(sc, wi, lohisign: int, idir: int, outflow: bool) -> np.ndarray:
    g = np.zeros(22)
    wi = np.ascontiguousarray(wi, dtype=np.float64)
    lib().tmko_edgebc(C.byref(sc.elastic), _dp(g), _dp(wi), lohisign, idir, int(outflow))
    return g


def rs_newton(sc, phi, psi, sn, a, V0guess):
    V = C.c_double(V0guess)
    tau = C.c_double(0.0)
    it = lib().tmko_rsnewton(C.byref(sc.elastic), C.byref(sc.rs), phi, psi, sn, a, C.byref(V),
                             C.byref(tau))
    return V.value, tau.value, it


def rs_fault(sc, wi, psi, x) -> np.ndarray:
    g = np.zeros(22)
    lib().tmko_rsfault(C.byref(sc.elastic), C.byref(sc.rs), _dp(g),
                       _dp(np.ascontiguousarray(wi, dtype=np.float64)), psi, x)
    return g


def sw_fault(sc, wi, b, xcell, g0=None) -> np.ndarray:
    g = np.zeros(22) if g0 is None else np.array(g0, dtype=np.float64)
    lib().tmko_swfault(C.byref(sc.elastic), C.byref(sc.sw), _dp(g),
                       _dp(np.ascontiguousarray(wi, dtype=np.float64)),
                       _dp(np.ascontiguousarray(b, dtype=np.float64)), xcell)
    return g


def plastic_flow(sc, s6l2, dt) -> np.ndarray:
    v = np.array(s6l2, dtype=np.float64)
    lib().tmko_plasticflow(C.byref(sc.elastic), C.byref(sc.plastic), _dp(v), dt)
    return v


# ------------------------------------------------------------- patch/level --
def patch_update_state(sc, U: np.ndarray, ulo, valid_lo, valid_hi, B: np.ndarray | None, bxlo: int,
                       time: float, dt: float, with_flux: bool = False):
    """LinElastPatchGodunov::updateState on a host FAB; U, B are updated in place.
    Returns (rc, Fx, Fy)."""
    assert U.shape[0] == 22
    uhi = (ulo[0] + U.shape[2] - 1, ulo[1] + U.shape[1] - 1)
    Fx = Fy = None
    if with_flux:
        nxv = valid_hi[0] - valid_lo[0] + 1
        nyv = valid_hi[1] - valid_lo[1] + 1
        Fx = np.zeros((22, nyv, nxv + 1))
        Fy = np.zeros((22, nyv + 1, nxv))
    bhi = bxlo + (B.shape[1] - 1 if B is not None else 0)
    rc = lib().tmko_patch_update_state(
        C.byref(sc.elastic), C.byref(sc.scheme), _ref(sc.rs), _ref(sc.sw), _dp(U), _iv(*ulo),
        _iv(*uhi), _dp(B), bxlo, bhi, _dp(Fx), _dp(Fy), _iv(*valid_lo), _iv(*valid_hi), _iv(0, 0),
        _iv(sc.nx - 1, sc.ny - 1), sc.dx, time, dt)
    return rc, Fx, Fy


def plastic_correction(sc, U: np.ndarray, ulo, blo, bhi, dt: float) -> None:
    uhi = (ulo[0] + U.shape[2] - 1, ulo[1] + U.shape[1] - 1)
    lib().tmko_plastic_correction(C.byref(sc.elastic), C.byref(sc.plastic), _dp(U), _iv(*ulo),
                                  _iv(*uhi), _iv(*blo), _iv(*bhi), dt)


def patch_update_state_3d(sc, U: np.ndarray, ulo, valid_lo, valid_hi, domain_lo, domain_hi,
                          B: np.ndarray | None, blo, dx: float, time: float, dt: float,
                          with_flux: bool = False):
    """LinElastPatchGodunov::updateState in 3-D on a host FAB U (22, nz, ny, nx)
    starting at cell ulo = (i, j, k); B (nb, nz_b, nx_b) the fault data on the
    domain's y-lo plane starting at blo = (i, k).  U, B are updated in place.
    Returns (rc, [F0, F1, F2]) with the face fluxes of the valid box."""
    assert U.shape[0] == 22 and U.ndim == 4
    uhi = (ulo[0] + U.shape[3] - 1, ulo[1] + U.shape[2] - 1, ulo[2] + U.shape[1] - 1)
    F = [None, None, None]
    if with_flux:
        n = [valid_hi[d] - valid_lo[d] + 1 for d in range(3)]
        for d in range(3):
            m = list(n)
            m[d] += 1
            F[d] = np.zeros((22, m[2], m[1], m[0]))
    if B is not None:
        bhi = (blo[0] + B.shape[2] - 1, blo[1] + B.shape[1] - 1)
    else:
        blo, bhi = (0, 0), (0, 0)
    rc = lib().tmko_patch_update_state_3d(
        C.byref(sc.elastic), C.byref(sc.scheme), _ref(sc.rs), _ref(sc.sw), _dp(U), _iv(*ulo), _iv(*uhi),
        _dp(B), _iv(*blo), _iv(*bhi), _dp(F[0]), _dp(F[1]), _dp(F[2]), _iv(*valid_lo), _iv(*valid_hi),
        _iv(*domain_lo), _iv(*domain_hi), dx, time, dt)
    return rc, F


def plastic_correction_3d(sc, U: np.ndarray, ulo, blo, bhi, dt: float) -> None:
    uhi = (ulo[0] + U.shape[3] - 1, ulo[1] + U.shape[2] - 1, ulo[2] + U.shape[1] - 1)
    lib().tmko_plastic_correction_3d(C.byref(sc.elastic), C.byref(sc.plastic), _dp(U), _iv(*ulo),
                                     _iv(*uhi), _iv(*blo), _iv(*bhi), dt)


def level_step(sc, Ug: np.ndarray, Bg: np.ndarray | None, boxes, time: float, dt: float,
               nthreads: int = 1, fric: np.ndarray | None = None) -> int:
    """LinElastLevelGodunov::step (+ plasticUpdate) for a single level whose
    patches `boxes` [(lo0, lo1, hi0, hi1), ...] tile the domain.  Ug is
    (22, ny+8, nx+8), Bg (nbdry, nx+8); both updated in place.  `fric` (3, nx+8):
    optional per-face rate-and-state a, b, L (an extension)."""
    flat = np.ascontiguousarray(np.array(boxes, dtype=np.int32).reshape(-1))
    F = None if fric is None else np.ascontiguousarray(fric, dtype=np.float64)
    return lib().tmko_level_step_fric(
        C.byref(sc.elastic), C.byref(sc.scheme), _ref(sc.rs), _ref(sc.sw), _ref(sc.plastic),
        _iv(0, 0), _iv(sc.nx - 1, sc.ny - 1), len(boxes), flat.ctypes.data_as(C.POINTER(C.c_int)),
        _dp(Ug), _dp(Bg), None if F is None else _dp(F), sc.dx, time, dt, nthreads)


# ------------------------------------------------------------------ AMR --
class LevelData:
    """A level as per-patch host arrays: U[p] (22, ny+8, nx+8) over the valid
    box grown by 4 ghosts, B[p] (nb, nx+8) for patches on the fault row, else
    None -- the layout of tetemoko_gb300.level.LinElastLevelGodunov's
    get_patch / set_patch."""

    def __init__(self, domain, dx: float, boxes, nb: int, U=None, B=None):
        self.domain = tuple(domain)
        self.dx = dx
        self.boxes = [tuple(b) for b in boxes]
        self.nb = nb
        g = A.TMK_NGHOST
        if U is None:
            U = [np.zeros((22, b[3] - b[1] + 1 + 2 * g, b[2] - b[0] + 1 + 2 * g)) for b in self.boxes]
        if B is None:
            B = [np.zeros((nb, b[2] - b[0] + 1 + 2 * g)) if self.fault(p) else None
                 for p, b in enumerate(self.boxes)]
        self.U = [np.ascontiguousarray(u, dtype=np.float64) for u in U]
        self.B = [None if b is None else np.ascontiguousarray(b, dtype=np.float64) for b in B]

    def fault(self, p) -> bool:
        return self.nb > 0 and self.boxes[p][1] == self.domain[1]

    def copy(self) -> "LevelData":
        return LevelData(self.domain, self.dx, self.boxes, self.nb, [u.copy() for u in self.U],
                         [None if b is None else b.copy() for b in self.B])

    def _pack(self):
        boxes = np.ascontiguousarray(np.array(self.boxes, dtype=np.int32).reshape(-1))
        U = np.concatenate([u.reshape(-1) for u in self.U])
        bl = [b.reshape(-1) for b in self.B if b is not None]
        B = np.concatenate(bl) if bl else None
        lv = _Level()
        for k in range(4):
            lv.dom[k] = self.domain[k]
        lv.dx = self.dx
        lv.npatch = len(self.boxes)
        lv.boxes = boxes.ctypes.data_as(C.POINTER(C.c_int))
        lv.U = _dp(U)
        lv.B = _dp(B)
        return lv, (boxes, U, B)

    def _unpack(self, keep):
        _, U, B = keep
        o = 0
        for u in self.U:
            u.reshape(-1)[:] = U[o:o + u.size]
            o += u.size
        o = 0
        for b in self.B:
            if b is not None:
                b.reshape(-1)[:] = B[o:o + b.size]
                o += b.size


def cf_fill(r: int, coarse_old: LevelData, coarse_new: LevelData, alpha: float, fine: LevelData) -> int:
    """Coarse-fine ghost fill of `fine` (in place)."""
    co, ko = coarse_old._pack()
    cn, kn = coarse_new._pack()
    f, kf = fine._pack()
    rc = lib().tmko_cf_fill(r, fine.nb, C.byref(co), C.byref(cn), alpha, C.byref(f))
    if rc == 0:
        fine._unpack(kf)
    return rc


def average_down(r: int, coarse: LevelData, fine: LevelData) -> int:
    c, kc = coarse._pack()
    f, kf = fine._pack()
    rc = lib().tmko_average_down(r, fine.nb, C.byref(c), C.byref(f))
    if rc == 0:
        coarse._unpack(kc)
    return rc


def fine_interp(r: int, coarse: LevelData, fine: LevelData) -> int:
    c, kc = coarse._pack()
    f, kf = fine._pack()
    rc = lib().tmko_fine_interp(r, fine.nb, C.byref(c), C.byref(f))
    if rc == 0:
        fine._unpack(kf)
    return rc


def tag_cells(sc, tp, fine: LevelData, coarse: LevelData | None = None, r: int = 2) -> np.ndarray:
    """AMRLevelLinElast::tagCells / tagCellsInit of `fine` (ghost cells filled
    in place): the tag mask over its domain, shape (ny, nx), uint8."""
    d = fine.domain
    mask = np.zeros((d[3] - d[1] + 1, d[2] - d[0] + 1), dtype=np.uint8)
    f, kf = fine._pack()
    c, kc = coarse._pack() if coarse is not None else (None, None)
    rc = lib().tmko_tag_cells(C.byref(sc.elastic), C.byref(sc.scheme), _ref(sc.rs), _ref(sc.sw), C.byref(tp), r,
                              C.byref(c) if c is not None else None, C.byref(f), mask.ctypes.data)
    assert rc == 0, rc
    fine._unpack(kf)
    return mask


def register_entries(r: int, coarse: LevelData, fine: LevelData) -> int:
    c, kc = coarse._pack()
    f, kf = fine._pack()
    n = C.c_int(0)
    assert lib().tmko_register_entries(r, C.byref(c), C.byref(f), C.byref(n)) == 0
    return n.value


def amr_run(sc, levels: list[LevelData], ratios, time: float, dt0: float, ncoarse: int, nthreads: int = 1) -> int:
    """`ncoarse` subcycled hierarchy steps (all levels updated in place)."""
    packed = [lv._pack() for lv in levels]
    arr = (_Level * len(levels))(*[p[0] for p in packed])
    rat = (C.c_int * max(1, len(ratios)))(*(list(ratios) or [1]))
    rc = lib().tmko_amr_run(C.byref(sc.elastic), C.byref(sc.scheme), _ref(sc.rs), _ref(sc.sw), _ref(sc.plastic),
                            len(levels), arr, rat, time, dt0, ncoarse, nthreads)
    for lv, (_, keep) in zip(levels, packed):
        lv._unpack(keep)
    return rc


def tile_boxes(nx: int, ny: int, max_grid: int):
    """Cover [0,nx)x[0,ny) with boxes of at most max_grid cells per side."""
    out = []
    for j0 in range(0, ny, max_grid):
        for i0 in range(0, nx, max_grid):
            out.append((i0, j0, min(i0 + max_grid, nx) - 1, min(j0 + max_grid, ny) - 1))
    return out


# ---------------------------------------------------------------- stations --
def station_cell(x: float, center: float, dx: float):
    """AMRLevelLinElast::define (srcLinElast/AMRLevelLinElast.cpp:260-335): the
    cell below a station and the distance from its centre (the reference's
    interpolation weight, not divided by dx)."""
    i = int(np.floor((x + center) / dx - 0.5))
    return i, -(i + 0.5) * dx + (x + center)


def station_values(domain, dx, Ug, Bg, fault_x, body_xy, center=(0.0, 0.0)):
    """AMRLevelLinElast::writeStationLevel (srcLinElast/AMRLevelLinElast.cpp:
    1758-1869) on domain-wide arrays (Ug (22, ny+8, nx+8), Bg (nb, nx+8)): one
    row of nb values per fault station, 22 per body station, in the
    reference's operation order."""
    g = A.TMK_NGHOST
    fault, body = [], []
    for x in fault_x:
        i, w = station_cell(x, center[0], dx)
        ci = i - domain[0] + g
        fault.append([Bg[c, ci] * (1 - w) + Bg[c, ci + 1] * w for c in range(Bg.shape[0])])
    for x, y in body_xy:
        i, wx = station_cell(x, center[0], dx)
        j, wy = station_cell(y, center[1], dx)
        ci, cj = i - domain[0] + g, j - domain[1] + g
        row = []
        for c in range(22):
            u = Ug[c]
            row.append(u[cj, ci] * (1 - wx) * (1 - wy) + u[cj, ci + 1] * wx * (1 - wy)
                       + u[cj + 1, ci] * (1 - wx) * wy + u[cj + 1, ci + 1] * wx * wy)
        body.append(row)
    return np.array(fault, dtype=np.float64).reshape(len(fault_x), -1), np.array(body, dtype=np.float64).reshape(
        len(body_xy), 22)
