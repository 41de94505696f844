"""Shared helpers of the test suite: seeded states and tolerances."""
from __future__ import annotations

import numpy as np

from tetemoko_gb300 import _capi as A

# FP64 parity tolerance against the oracle: 1e-12 relative
RTOL_FP64 = 1e-12


def perturbed_state(sc, rng, lo=(0, 0), hi=None, amp_v=0.5, amp_s=5.0, smooth=True):
    """Background state plus seeded smooth + rough perturbations (all 22 comps
    but lambda, gamma) over [lo, hi] grown by the ghost width."""
    U = sc.initial_U(lo=lo, hi=hi)
    ny, nx = U.shape[1:]
    y, x = np.mgrid[0:ny, 0:nx]
    for c in range(22):
        k = c % 11
        if k in (9, 10):
            continue
        amp = amp_v if k < 3 else amp_s
        f = np.zeros((ny, nx))
        if smooth:
            for _ in range(3):
                kx, ky = rng.uniform(0.05, 0.5, 2)
                ph = rng.uniform(0, 2 * np.pi)
                f += np.sin(kx * x + ky * y + ph)
        f += 0.3 * rng.standard_normal((ny, nx))
        U[c] += amp * f / 3.0
    return U


def rel_err(a, b):
    """max |a-b| / max|b| per component (leading axis), max over components."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    a2 = a.reshape(a.shape[0], -1)
    b2 = b.reshape(b.shape[0], -1)
    # components that are zero in the reference are measured against 1e-6 of
    # the largest component, so that they must stay (nearly) zero too
    scale = np.maximum(np.abs(b2).max(axis=1), 1e-6 * max(np.abs(b2).max(), 1e-300))
    return float((np.abs(a2 - b2).max(axis=1) / scale).max())


def perturbed_state_3d(sc, rng, lo, hi, ghost=4, amp_v=0.5, amp_s=5.0):
    """3-D state FAB (22, nz, ny, nx) over [lo, hi] grown by `ghost`: the
    background plus seeded smooth and rough perturbations (lambda, gamma kept)."""
    n = [hi[d] - lo[d] + 1 + 2 * ghost for d in range(3)]
    U = np.empty((22, n[2], n[1], n[0]))
    U[:] = sc.background()[:, None, None, None]
    z, y, x = np.mgrid[0:n[2], 0:n[1], 0:n[0]]
    for c in range(22):
        k = c % 11
        if k in (9, 10):
            continue
        amp = amp_v if k < 3 else amp_s
        f = np.zeros(U.shape[1:])
        for _ in range(3):
            kx, ky, kz = rng.uniform(0.05, 0.5, 3)
            f += np.sin(kx * x + ky * y + kz * z + rng.uniform(0, 2 * np.pi))
        f += 0.3 * rng.standard_normal(U.shape[1:])
        U[c] += amp * f / 3.0
    return U


def random_B_3d(sc, rng, nx, nz):
    """Fault data (nb, nz, nx) from the scenario's initial values with seeded
    state (rate and state) or slip (slip weakening)."""
    B1 = sc.initial_B(xlo=0, xhi=nx - 1, ghost=0)
    B = np.repeat(B1[:, None, :], nz, axis=1).copy()
    if sc.scheme.fault_law == A.TMK_FAULT_RS:
        B[10] += 0.02 * rng.standard_normal((nz, nx))
        B[8] = np.abs(rng.standard_normal((nz, nx)))
    else:
        B[7] = 0.3 * np.abs(rng.standard_normal((nz, nx)))
    return B
