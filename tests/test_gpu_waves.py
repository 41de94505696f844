"""The plane-wave known answers of test_oracle_waves.py on the GPU: the FP64
form equals the oracle's step on them, and the mixed form (FP32 volume) reaches
the exact solution at the same second-order rate, its FP32 rounding below the
truncation error on these grids."""
import math

import numpy as np
import pytest

from tetemoko_gb300 import _capi as A
from tests import test_oracle_waves as W

pytestmark = pytest.mark.gpu
G = A.TMK_NGHOST


def _gpu_error(n: int, along: str, wave: str, prec: int) -> float:
    from tetemoko_gb300.level import Context, LinElastLevelGodunov
    sc = W._scenario(n, along, wave)
    sc.scheme.precision = prec
    U = W._wave_state(sc, along, wave, 0.0)
    speed = sc.elastic.cp if wave == "P" else sc.elastic.cs
    steps = int(math.ceil(W.TRAVEL / (speed * sc.dt())))
    dt = W.TRAVEL / (speed * steps)
    ctx = Context(sc)
    lvl = LinElastLevelGodunov(ctx, [(0, 0, sc.nx - 1, sc.ny - 1)])
    lvl.set_level(U, None)
    t = 0.0
    for _ in range(steps):
        lvl.step(t, dt)
        t += dt
    out = U.copy()
    lvl.get_level(out, None)
    assert lvl.status()[0] == 0
    lvl.close()
    ctx.close()
    exact = W._wave_state(sc, along, wave, t)
    comp = (3 if along == "x" else 4) if wave == "P" else 6
    if along == "x":
        j = G + sc.ny // 2
        got, ref = out[comp, j, G:-G], exact[comp, j, G:-G]
    else:
        i = G + sc.nx // 2
        got, ref = out[comp, G:-G, i], exact[comp, G:-G, i]
    return float(np.sum(np.abs(got - ref)) * sc.dx / (W.AMP * W.WIDTH))


@pytest.mark.parametrize("along,wave", [("x", "P"), ("y", "S")])
def test_mixed_form_converges_like_the_oracle(cuda_lib, along, wave):
    mixed = [_gpu_error(n, along, wave, A.TMK_PREC_MIXED) for n in (64, 128, 256)]
    fp64 = _gpu_error(256, along, wave, A.TMK_PREC_FP64)
    ref = W._error(256, along, wave)
    orders = [math.log2(mixed[k] / mixed[k + 1]) for k in range(2)]
    print(f"{wave} along {along}: mixed L1 errors {['%.3e' % e for e in mixed]}, orders "
          f"{['%.2f' % o for o in orders]}; FP64 GPU {fp64:.3e}, oracle {ref:.3e}")
    # the FP64 form is the oracle's step to ~1e-11 relative per component (a
    # 70 MPa shear background carries the S pulse), far below the error measured
    assert abs(fp64 - ref) <= 1e-6 * ref
    assert orders[1] > 1.6
    # FP32 state rounding of the pulse on that background, ~4e-6 MPa a step
    assert abs(mixed[2] - ref) <= 0.15 * ref


@pytest.mark.parametrize("prec", [A.TMK_PREC_FP64, A.TMK_PREC_MIXED], ids=["fp64", "mixed"])
def test_uniformly_sliding_fault_on_the_gpu(cuda_lib, prec):
    """The exact slip rate, traction and slip of a uniformly sliding
    slip-weakening fault (test_oracle_waves.py): the FP64 form to rounding, the
    mixed form to FP32 rounding of the 80 MPa stresses."""
    from tetemoko_gb300.level import Context, LinElastLevelGodunov
    sc = W.uniform_sliding_scenario(prec)
    V, tau_d = W.uniform_sliding_answer(sc)
    U, B = sc.initial_U(), sc.initial_B()
    ctx = Context(sc)
    lvl = LinElastLevelGodunov(ctx, [(0, 0, 31, 15), (32, 0, 63, 15), (0, 16, 63, 31)])
    lvl.set_level(U, B)
    dt = sc.dt()
    for k in range(12):
        lvl.step(k * dt, dt)
    lvl.get_level(U, B)
    assert lvl.status()[0] == 0
    lvl.close()
    ctx.close()
    t = 12 * dt
    tol = 1e-12 if prec == A.TMK_PREC_FP64 else 1e-5
    mid = slice(G + 24, G + 40)
    np.testing.assert_allclose(B[4, mid], V, rtol=tol)
    np.testing.assert_allclose(B[2, mid], tau_d, rtol=tol)
    np.testing.assert_allclose(B[5, mid], V * t, rtol=tol)
    np.testing.assert_allclose(U[6, G, mid], tau_d, atol=0.01 * (sc.elastic.sxy0 - tau_d))


@pytest.mark.parametrize("prec", [A.TMK_PREC_FP64, A.TMK_PREC_MIXED], ids=["fp64", "mixed"])
def test_uniformly_sliding_rate_and_state_fault_on_the_gpu(cuda_lib, prec):
    """The uniformly sliding rate-and-state fault of test_oracle_waves.py on
    three patches: slip rate (component 2) against its ODE at the step's
    midpoint and state (10) at the step's end after 20, 40 and 60 steps; the
    FP64 form to the oracle's 1e-5 / 1e-6, the mixed form (FP32 volume
    stresses near 70 MPa) to 1e-4 / 1e-5."""
    from tetemoko_gb300.level import Context, LinElastLevelGodunov
    sc = W.uniform_rs_scenario(prec)
    U, B = sc.initial_U(), sc.initial_B()
    dt = sc.dt()
    V_ode, psi_ode = W.uniform_rs_answer(sc, 61 * dt)
    ctx = Context(sc)
    lvl = LinElastLevelGodunov(ctx, [(0, 0, 63, 31), (64, 0, 127, 31), (0, 32, 127, 63)])
    lvl.set_level(U, B)
    c = G + sc.nx // 2
    tv, tp = (1e-5, 1e-6) if prec == A.TMK_PREC_FP64 else (1e-4, 1e-5)
    for k in range(60):
        lvl.step(k * dt, dt)
        if (k + 1) % 20 == 0:
            t = (k + 1) * dt
            lvl.get_level(U, B)
            assert lvl.status()[0] == 0
            V = V_ode(t - 0.5 * dt)
            assert abs(B[2, c] - V) <= tv * V, (t, B[2, c], V)
            assert abs(B[10, c] - psi_ode(t)) <= tp, (t, B[10, c], psi_ode(t))
    lvl.close()
    ctx.close()
