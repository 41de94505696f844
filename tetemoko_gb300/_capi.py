"""ctypes mirror of include/tetemoko_gb300.h and the loader of the CUDA library.

The structs here are the C ABI's POD types; importing this module never loads
the CUDA library.  `lib()` loads `libtetemoko_gb300.so` from this package
directory and raises if it is missing: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

TMK_NCOMP = 22
TMK_RS_NBDRY = 11
TMK_SW_NBDRY = 9
TMK_NGHOST = 4
TMK_SW_MAX_PATCHES = 8

TMK_OK = 0
STATUS_NAMES = {
    0: "TMK_OK", 1: "TMK_ERR_BAD_DESC", 2: "TMK_ERR_NAN_STATE", 3: "TMK_ERR_TIMEOUT",
    4: "TMK_ERR_CUDA", 5: "TMK_ERR_UNSUPPORTED", 6: "TMK_ERR_ALLOC", 7: "TMK_ERR_NO_DEVICE",
    8: "TMK_ERR_TOO_LARGE",
}
TMK_ERR_TOO_LARGE = 8
TMK_NOALLOC_SCRATCH_BYTES = 8 << 20

TMK_BC_OUTFLOW, TMK_BC_FREE, TMK_BC_FAULT = 0, 1, 2
TMK_FAULT_NONE, TMK_FAULT_RS, TMK_FAULT_SW = 0, 1, 2
TMK_RS_SLIP_LAW, TMK_RS_AGING_LAW = 0, 1
TMK_SW_LAYOUT_REFERENCE9, TMK_SW_LAYOUT_OFFSET11 = 0, 1
TMK_PREC_FP64, TMK_PREC_MIXED = 0, 1


class ElasticParams(C.Structure):
    _fields_ = [("cs", C.c_double), ("cp", C.c_double), ("G", C.c_double), ("rho", C.c_double),
                ("sxx0", C.c_double), ("syy0", C.c_double), ("szz0", C.c_double),
                ("sxy0", C.c_double), ("sxz0", C.c_double), ("syz0", C.c_double)]


class RSParams(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "r0", "x0", "y0", "nsig", "ntime", "a", "b", "V0", "f0", "L", "fw", "Vw", "fexp",
        "ramp_x", "ramp_w", "ramp_a", "ramp_Vw", "rupture_threshold", "psi_init")] + [
        ("state_law", C.c_int)]


_P = TMK_SW_MAX_PATCHES


class SWParams(C.Structure):
    _fields_ = [("fs", C.c_double), ("fd", C.c_double), ("dw", C.c_double), ("smooth", C.c_double),
                ("num_patches", C.c_int),
                ("xc", C.c_double * _P), ("xw", C.c_double * _P), ("zc", C.c_double * _P),
                ("zw", C.c_double * _P), ("tau", C.c_double * _P),
                ("fric_box_center", C.c_double * 2), ("fric_box_width", C.c_double * 2),
                ("outside_friction", C.c_double), ("rupture_threshold", C.c_double),
                ("layout", C.c_int)]


class PlasticParams(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("mu", "beta", "eta", "b", "h")]


class Scheme(C.Structure):
    _fields_ = [("normal_pred_order", C.c_int), ("use_prim_limiting", C.c_int),
                ("use_char_limiting", C.c_int), ("boundary_type", C.c_int * 6),
                ("fault_law", C.c_int), ("plasticity", C.c_int), ("precision", C.c_int),
                ("volume_kernel", C.c_int), ("use_fourth_order_slopes", C.c_int)]


TMK_VOLUME_AUTO, TMK_VOLUME_TILE, TMK_VOLUME_MARCH = 0, 1, 2


class Tuning(C.Structure):
    _fields_ = [("volume_kernel", C.c_int), ("march_waves", C.c_int * 2), ("min_run", C.c_int),
                ("fault_displace", C.c_int), ("fault_seg", C.c_int), ("fault_first", C.c_int),
                ("plastic_fused", C.c_int)]

    def as_dict(self) -> dict:
        return {"volume_kernel": {TMK_VOLUME_MARCH: "march", TMK_VOLUME_TILE: "tile"}.get(self.volume_kernel),
                "march_waves": list(self.march_waves), "min_run": self.min_run,
                "fault_displace": self.fault_displace, "fault_seg": self.fault_seg,
                "fault_first": self.fault_first, "plastic_fused": self.plastic_fused}


class TagParams(C.Structure):
    _fields_ = [("level", C.c_int), ("initial", C.c_int), ("refine_thresh", C.c_double),
                ("plastic_thresh", C.c_double), ("tag_buffer", C.c_int), ("x_coarsen", C.c_double * 2),
                ("y_coarsen", C.c_double * 2), ("slope_coarsen", C.c_double), ("width_coarsen", C.c_double),
                ("x_coarsen2", C.c_double * 2), ("y_coarsen2", C.c_double * 2), ("coarsen2_max_level", C.c_int),
                ("slip_rate_thresh", C.c_double)]


def tag_params(level=0, initial=False, refine_thresh=0.01, plastic_thresh=1e-5, tag_buffer=2,
               x_coarsen=(-1e40, 1e40), y_coarsen=(-1e40, 1e40), slope_coarsen=0.0, width_coarsen=1e40,
               x_coarsen2=(-1e40, 1e40), y_coarsen2=(-1e40, 1e40), coarsen2_max_level=100,
               slip_rate_thresh=0.0) -> TagParams:
    """Tagging parameters with the input deck's defaults (execLinElast/amrGodunov.cpp:274-283, 400-440);
    slip_rate_thresh > 0 adds the slip-rate tag of the fault row (an extension)."""
    t = TagParams()
    t.level, t.initial, t.refine_thresh, t.plastic_thresh = level, int(initial), refine_thresh, plastic_thresh
    t.tag_buffer, t.slope_coarsen, t.width_coarsen = tag_buffer, slope_coarsen, width_coarsen
    t.x_coarsen[:] = list(x_coarsen)
    t.y_coarsen[:] = list(y_coarsen)
    t.x_coarsen2[:] = list(x_coarsen2)
    t.y_coarsen2[:] = list(y_coarsen2)
    t.coarsen2_max_level = coarsen2_max_level
    t.slip_rate_thresh = slip_rate_thresh
    return t


class Fab(C.Structure):
    _fields_ = [("data", C.c_void_p), ("lo", C.c_int * 2), ("hi", C.c_int * 2), ("ncomp", C.c_int)]


class Box(C.Structure):
    _fields_ = [("lo", C.c_int * 2), ("hi", C.c_int * 2)]


def box(lo0, lo1, hi0, hi1) -> Box:
    b = Box()
    b.lo[0], b.lo[1], b.hi[0], b.hi[1] = lo0, lo1, hi0, hi1
    return b


class Fab3(C.Structure):
    _fields_ = [("data", C.c_void_p), ("lo", C.c_int * 3), ("hi", C.c_int * 3), ("ncomp", C.c_int)]


class Box3(C.Structure):
    _fields_ = [("lo", C.c_int * 3), ("hi", C.c_int * 3)]


def box3(lo, hi) -> Box3:
    b = Box3()
    for d in range(3):
        b.lo[d], b.hi[d] = lo[d], hi[d]
    return b


LIBNAME = "libtetemoko_gb300.so"
_lib = None


def lib_path() -> str:
    return os.path.join(os.path.dirname(os.path.abspath(__file__)), LIBNAME)


def lib() -> C.CDLL:
    """Load the CUDA library (built in-tree by tetemoko_gb300.build)."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not os.path.exists(path):
        raise RuntimeError(
            f"{LIBNAME} is not built (expected at {path}); run "
            "`python -c 'import __graft_entry__ as g; g.build()'`. There is no CPU fallback.")
    L = C.CDLL(path)
    vp, ip, dp = C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_double)
    L.tmk_abi_version.restype = C.c_int
    L.tmk_context_create.argtypes = [C.POINTER(ElasticParams), C.POINTER(Scheme), C.POINTER(RSParams),
                                     C.POINTER(SWParams), C.POINTER(PlasticParams), C.POINTER(vp)]
    L.tmk_context_destroy.argtypes = [vp]
    L.tmk_context_destroy.restype = None
    L.tmk_context_constants.argtypes = [vp, dp]
    L.tmk_patch_update_state.argtypes = [vp, C.POINTER(Fab), C.POINTER(Fab), C.POINTER(Fab), C.POINTER(Fab),
                                         C.POINTER(Box), C.POINTER(Box), C.c_double, C.c_double, C.c_double,
                                         dp, vp]
    L.tmk_patch_update_state_noalloc.argtypes = L.tmk_patch_update_state.argtypes
    L.tmk_patch_update_state_noalloc.restype = C.c_int
    L.tmk_plastic_update.argtypes = [vp, C.POINTER(Fab), C.POINTER(Box), C.c_double, vp]
    L.tmk_max_wave_speed.argtypes = [vp, dp]
    F3 = C.POINTER(Fab3)
    L.tmk_patch_update_state_3d.argtypes = [vp, F3, F3, F3, F3, F3, C.POINTER(Box3), C.POINTER(Box3), C.c_double,
                                            C.c_double, C.c_double, dp, vp]
    L.tmk_plastic_update_3d.argtypes = [vp, F3, C.POINTER(Box3), C.c_double, vp]
    L.tmk_patches_update_state_3d.argtypes = [vp, C.c_int, F3, F3, F3, F3, F3, C.POINTER(Box3), C.POINTER(Box3),
                                              C.c_double, C.c_double, C.c_double, dp, vp]
    L.tmk_level3d_create.argtypes = [vp, C.POINTER(Box3), C.c_double, C.c_int, C.POINTER(Box3), C.POINTER(vp)]
    L.tmk_level3d_destroy.argtypes = [vp]
    L.tmk_level3d_destroy.restype = None
    L.tmk_level3d_set_patch.argtypes = [vp, C.c_int, vp, vp, C.c_int]
    L.tmk_level3d_get_patch.argtypes = [vp, C.c_int, vp, vp, C.c_int]
    L.tmk_level3d_patch_fabs.argtypes = [vp, C.c_int, F3, F3]
    L.tmk_level3d_exchange.argtypes = [vp, vp]
    L.tmk_level3d_step.argtypes = [vp, C.c_double, C.c_double, dp, vp]
    L.tmk_level_create.argtypes = [vp, C.POINTER(Box), C.c_double, C.c_int, C.POINTER(Box), C.POINTER(vp)]
    L.tmk_level_destroy.argtypes = [vp]
    L.tmk_level_get_tuning.argtypes = [vp, C.POINTER(Tuning)]
    L.tmk_level_set_tuning.argtypes = [vp, C.POINTER(Tuning)]
    L.tmk_amr_autotune.argtypes = [vp, C.c_double, C.c_int, vp, C.POINTER(Tuning), dp]
    L.tmk_level_autotune.argtypes = [vp, C.c_double, C.c_double, C.c_int, vp, C.POINTER(Tuning), dp]
    L.tmk_stations_create.argtypes = [vp, C.c_int, dp, C.c_int, dp, dp, dp, C.c_int, C.POINTER(vp)]
    L.tmk_stations_destroy.argtypes = [vp]
    L.tmk_stations_destroy.restype = None
    L.tmk_stations_record.argtypes = [vp, C.c_double, vp]
    L.tmk_stations_layout.argtypes = [vp, ip, ip]
    L.tmk_stations_read.argtypes = [vp, dp, C.c_int, ip, C.POINTER(C.c_longlong)]
    L.tmk_level_attach_stations.argtypes = [vp, vp]
    L.tmk_level_tag_cells.argtypes = [vp, C.POINTER(TagParams), vp, C.c_int, vp]
    L.tmk_level_set_fault_friction.argtypes = [vp, C.c_int, vp, C.c_int]
    L.tmk_level_get_fault_friction.argtypes = [vp, C.c_int, vp, C.c_int, ip]
    L.tmk_ensemble_create.argtypes = [C.c_int, C.POINTER(vp), C.POINTER(Box), C.c_double, C.c_int,
                                      C.POINTER(Box), ip, C.POINTER(vp)]
    L.tmk_level_destroy.restype = None
    L.tmk_level_set_patch.argtypes = [vp, C.c_int, vp, vp, C.c_int]
    L.tmk_level_get_patch.argtypes = [vp, C.c_int, vp, vp, C.c_int]
    L.tmk_level_put_valid.argtypes = [vp, C.c_int, vp, vp, C.c_int]
    L.tmk_level_take_valid.argtypes = [vp, C.c_int, vp, vp, C.c_int]
    L.tmk_level_step.argtypes = [vp, C.c_double, C.c_double, vp, dp]
    L.tmk_level_status.argtypes = [vp, C.POINTER(C.c_longlong)]
    L.tmk_level_launches_per_step.argtypes = [vp]
    L.tmk_level_launches_per_step.restype = C.c_int
    L.tmk_level_profile.argtypes = [vp, C.c_int, C.c_int]
    L.tmk_level_profile_read.argtypes = [vp, dp, ip]
    L.tmk_level_step_cf.argtypes = [vp, C.c_double, C.c_double, C.c_double, C.c_double, vp, dp]
    L.tmk_level_attach_coarser.argtypes = [vp, vp, C.c_int]
    L.tmk_level_detach_coarser.argtypes = [vp]
    L.tmk_level_fill_coarse_fine.argtypes = [vp, C.c_double, vp]
    L.tmk_level_reflux.argtypes = [vp, vp]
    L.tmk_level_average_down.argtypes = [vp, vp]
    L.tmk_level_interp_from_coarser.argtypes = [vp, vp]
    L.tmk_level_copy_overlap.argtypes = [vp, vp, vp]
    L.tmk_level_register_size.argtypes = [vp, ip]
    L.tmk_amr_create.argtypes = [C.c_int, C.POINTER(vp), ip, C.c_double, C.POINTER(vp)]
    L.tmk_amr_destroy.argtypes = [vp]
    L.tmk_amr_destroy.restype = None
    L.tmk_amr_step.argtypes = [vp, C.c_double, vp]
    L.tmk_amr_time.argtypes = [vp, C.c_int, dp]
    L.tmk_amr_cell_updates.argtypes = [vp]
    L.tmk_amr_cell_updates.restype = C.c_longlong
    L.tmk_amr_launches_per_step.argtypes = [vp]
    L.tmk_amr_launches_per_step.restype = C.c_int
    L.tmk_level_graph_create.argtypes = [vp, C.c_int, C.c_double, C.c_double, C.POINTER(vp)]
    L.tmk_amr_graph_create.argtypes = [vp, C.c_int, C.c_double, C.POINTER(vp)]
    L.tmk_graph_launch.argtypes = [vp, C.c_double, vp]
    L.tmk_graph_destroy.argtypes = [vp]
    L.tmk_graph_destroy.restype = None
    for name in ("tmk_context_create", "tmk_context_constants", "tmk_patch_update_state",
                 "tmk_plastic_update", "tmk_max_wave_speed", "tmk_level_create", "tmk_level_set_patch",
                 "tmk_level_get_patch", "tmk_level_step", "tmk_level_status", "tmk_level_profile",
                 "tmk_level_profile_read", "tmk_level_step_cf", "tmk_level_attach_coarser",
                 "tmk_level_detach_coarser", "tmk_level_fill_coarse_fine", "tmk_level_reflux",
                 "tmk_level_average_down", "tmk_level_interp_from_coarser", "tmk_level_copy_overlap",
                 "tmk_level_register_size", "tmk_amr_create", "tmk_amr_step", "tmk_amr_time",
                 "tmk_level_graph_create", "tmk_amr_graph_create", "tmk_graph_launch",
                 "tmk_patch_update_state_3d", "tmk_plastic_update_3d", "tmk_patches_update_state_3d"):
        getattr(L, name).restype = C.c_int
    _lib = L
    return L


class TmkError(RuntimeError):
    def __init__(self, code: int, where: str):
        super().__init__(f"{where}: {STATUS_NAMES.get(code, code)}")
        self.code = code


def check(code: int, where: str) -> None:
    if code != TMK_OK:
        raise TmkError(code, where)
