"""The oracle's 3-D patch step (CH_SPACEDIM == 3) against properties of the
3-D corner transport upwind scheme:
  * a state that does not vary in z, on a patch away from the z edges of the
    domain, gives exactly the 2-D step (every z correction is a difference of
    equal face states), except on the fault row, where the 3-D scheme's
    (1/3) dt boundary-data prediction enters;
  * without a fault the step commutes with the mirror exchanging x and z, to
    rounding (the transverse corrections are added in another order);
  * the 3-D plastic correction is the pointwise 2-D one."""
import numpy as np
import pytest

import oracle as O
from tetemoko_gb300 import _capi as A
from tetemoko_gb300 import scenarios as S

from helpers import perturbed_state, perturbed_state_3d, rel_err

G = A.TMK_NGHOST


def _no_fault(sc):
    sc.scheme.fault_law = A.TMK_FAULT_NONE
    sc.scheme.boundary_type[2] = A.TMK_BC_FREE
    return sc


CASES = [
    ("none_ppm", lambda: _no_fault(S.rate_state(nx=24, ny=16, dx=0.1))),
    ("rs_ppm", lambda: S.rate_state(nx=24, ny=16, dx=0.1)),
    ("sw_ppm", lambda: S.slip_weakening(nx=24, ny=16, dx=0.1)),
    ("sw_ref9_charlim", lambda: _charlim(S.slip_weakening(nx=24, ny=16, dx=0.1,
                                                            layout=A.TMK_SW_LAYOUT_REFERENCE9))),
    ("rs_plm4", lambda: _plm(S.rate_state(nx=24, ny=16, dx=0.1))),
    ("none_ctu", lambda: _ctu(_no_fault(S.rate_state(nx=24, ny=16, dx=0.1)))),
]


def _charlim(sc):
    sc.scheme.use_prim_limiting, sc.scheme.use_char_limiting = 0, 1
    return sc


def _plm(sc):
    sc.scheme.normal_pred_order = 1
    return sc


def _ctu(sc):
    sc.scheme.normal_pred_order = 0
    return sc


@pytest.mark.parametrize("name,make", CASES, ids=[c[0] for c in CASES])
@pytest.mark.parametrize("valid", [(0, 0, 23, 15), (3, 2, 20, 12)], ids=["whole", "inner"])
def test_z_uniform_state_reduces_to_2d(name, make, valid):
    sc = make()
    rng = np.random.default_rng(7)
    U2 = perturbed_state(sc, rng, lo=valid[:2], hi=valid[2:])
    ulo2 = (valid[0] - G, valid[1] - G)
    fault = sc.scheme.fault_law != A.TMK_FAULT_NONE
    B2 = None
    if fault:
        B2 = sc.initial_B(xlo=valid[0], xhi=valid[2])
        if sc.scheme.fault_law == A.TMK_FAULT_RS:
            B2[10] += 0.02 * rng.standard_normal(B2.shape[1])
        else:
            B2[7] = 0.3 * np.abs(rng.standard_normal(B2.shape[1]))
    dt, t = sc.dt(), 1.25
    Ur, Br = U2.copy(), None if B2 is None else B2.copy()
    rc, Fx, Fy = O.patch_update_state(sc, Ur, ulo2, valid[:2], valid[2:], Br, valid[0] - G, t, dt, with_flux=True)
    assert rc == 0
    klo, khi, nz = 2, 3, 6
    U3 = np.repeat(U2[:, None], khi - klo + 1 + 2 * G, axis=1).copy()
    B3 = None if B2 is None else np.repeat(B2[:, None], khi - klo + 1 + 2 * G, axis=1).copy()
    rc3, F = O.patch_update_state_3d(sc, U3, (ulo2[0], ulo2[1], klo - G), (valid[0], valid[1], klo),
                                     (valid[2], valid[3], khi), (0, 0, 0), (sc.nx - 1, sc.ny - 1, nz - 1),
                                     B3, (valid[0] - G, klo - G), sc.dx, t, dt, with_flux=True)
    assert rc3 == 0
    rows = slice(G + 1 if (fault and valid[1] == 0) else 0, None)
    for kk in range(G, G + khi - klo + 1):
        assert np.array_equal(U3[:, kk][:, rows], Ur[:, rows])
        # the z fluxes of a z-uniform state have no divergence
        assert np.array_equal(F[2][:, kk - G + 1], F[2][:, kk - G])
    fr = slice(1 if (fault and valid[1] == 0) else 0, None)
    assert np.array_equal(F[0][:, 0][:, fr], Fx[:, fr])
    if fault and valid[1] == 0:
        # the fault row moves by the 3-D predictor's boundary data only
        assert rel_err(U3[:, G, G], Ur[:, G]) < 0.05
        assert not np.array_equal(B3[:, G], Br)


def _mirror_xz(U):
    """State FAB (22, nz, ny, nx) mirrored by x <-> z: components permuted
    (vx<->vz, sxx<->szz, sxy<->syz) and axes exchanged."""
    perm = [2, 1, 0, 5, 4, 3, 8, 7, 6, 9, 10]
    perm = perm + [11 + p for p in perm]
    return np.ascontiguousarray(U[perm].transpose(0, 3, 2, 1))


@pytest.mark.parametrize("order", [2, 1, 0])
def test_no_fault_step_commutes_with_xz_mirror(order):
    sc = _no_fault(S.rate_state(nx=10, ny=9, dx=0.1))
    sc.scheme.normal_pred_order = order
    for k in range(6):
        sc.scheme.boundary_type[k] = (0, 1, 1, 0, 0, 1)[k]
    # the mirror exchanges the x and z boundary types
    rng = np.random.default_rng(11)
    lo, hi = (1, 0, 2), (8, 6, 7)
    dom_lo, dom_hi = (0, 0, 0), (9, 8, 9)
    U = perturbed_state_3d(sc, rng, lo, hi)
    dt = 0.5 * sc.dt()
    Ua = U.copy()
    rc, Fa = O.patch_update_state_3d(sc, Ua, tuple(l - G for l in lo), lo, hi, dom_lo, dom_hi, None, (0, 0),
                                     sc.dx, 0.0, dt, with_flux=True)
    assert rc == 0
    scm = _no_fault(S.rate_state(nx=10, ny=9, dx=0.1))
    scm.scheme.normal_pred_order = order
    for k, v in enumerate((0, 1, 1, 0, 0, 1)):
        scm.scheme.boundary_type[k] = v
    scm.scheme.boundary_type[0], scm.scheme.boundary_type[4] = sc.scheme.boundary_type[4], sc.scheme.boundary_type[0]
    scm.scheme.boundary_type[1], scm.scheme.boundary_type[5] = sc.scheme.boundary_type[5], sc.scheme.boundary_type[1]
    e = scm.elastic
    e.sxx0, e.szz0 = sc.elastic.szz0, sc.elastic.sxx0
    e.sxy0, e.syz0 = sc.elastic.syz0, sc.elastic.sxy0
    Um = _mirror_xz(U)
    rc, Fm = O.patch_update_state_3d(scm, Um, (lo[2] - G, lo[1] - G, lo[0] - G), (lo[2], lo[1], lo[0]),
                                     (hi[2], hi[1], hi[0]), dom_lo, (9, 8, 9), None, (0, 0), scm.dx, 0.0, dt,
                                     with_flux=True)
    assert rc == 0
    v = (slice(None), slice(G, -G), slice(G, -G), slice(G, -G))
    assert rel_err(_mirror_xz(Ua)[v], Um[v]) < 1e-12
    assert rel_err(_mirror_xz(Fa[0]), Fm[2]) < 1e-12


def test_plastic_correction_3d_is_pointwise():
    sc = S.slip_weakening(nx=8, ny=8, dx=0.1, plasticity=True)
    rng = np.random.default_rng(3)
    U = perturbed_state_3d(sc, rng, (0, 0, 0), (5, 4, 3), amp_s=60.0)
    U3 = U.copy()
    O.plastic_correction_3d(sc, U3, (-G, -G, -G), (0, 0, 0), (5, 4, 3), 0.01)
    for k in range(G, G + 4):
        U2 = np.ascontiguousarray(U[:, k])
        O.plastic_correction(sc, U2, (-G, -G), (0, 0), (5, 4), 0.01)
        assert np.array_equal(U3[:, k], U2)
    assert not np.array_equal(U3, U)
