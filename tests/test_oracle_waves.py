"""Known answers of the elastic wave equation for the oracle's level step.

A smooth plane P wave travelling along x and a plane S wave travelling along y
(no fault, absorbing edges) are advanced by the oracle's LinElastLevelGodunov
step and compared with the exact solution, the initial pulse translated by the
wave speed: the error must fall at close to second order as the grid is
refined (PPM with primitive limiting, corner transport upwind).  The comparison
row (column) lies outside the region the domain edges reach in the time run.
The plain FP64 GPU form equals the oracle step for step (test_gpu_march.py,
test_gpu_parity.py), so these answers pin it as well.

For a wave f travelling in +d along direction d with speed c and impedance
Z = rho c the equations v_t = (1/rho) div(sigma), sigma_t = C : grad(v) give
sigma_dd = f(x_d - c t), v_d = -sigma_dd / Z (P wave; sigma of the two other
normal directions = lam/(lam+2G) sigma_dd), and sigma_de = f, v_e = -f / Zs for
an S wave polarised along e.
"""
import math

import numpy as np
import pytest

import oracle as O
from tetemoko_gb300 import _capi as A, scenarios as S

G = A.TMK_NGHOST
AMP = 1.0          # MPa
WIDTH = 0.8        # km, Gaussian half-width of the pulse
TRAVEL = 2.0       # km the pulse travels
LEN = 12.8         # km along the wave
# km across it: the side edges send P waves inward (an S wave's particle
# velocity crosses them) at cp during the pulse's travel time; the comparison
# row (column) in the middle must stay beyond their reach
SIDE = {"P": 6.0, "S": 9.0}


def _scenario(n: int, along: str, wave: str):
    dx = LEN / n
    m = int(round(SIDE[wave] / dx))
    nx, ny = (n, m) if along == "x" else (m, n)
    return S.Scenario(name="plane_wave", nx=nx, ny=ny, dx=dx, cfl=0.9, elastic=S._elastic(),
                      scheme=S._scheme(A.TMK_FAULT_NONE, bc=(0, 0, 0, 0, 0, 0)))


def _pulse(s: np.ndarray) -> np.ndarray:
    return AMP * np.exp(-(s / WIDTH) ** 2)


def _wave_state(sc, along: str, wave: str, t: float) -> np.ndarray:
    """The state at time t (cell centres), ghosts included."""
    c = sc.constants()
    e = sc.elastic
    U = sc.initial_U()
    xs = (np.arange(sc.nx + 2 * G) - G + 0.5) * sc.dx
    ys = (np.arange(sc.ny + 2 * G) - G + 0.5) * sc.dx
    pos = (xs[None, :] if along == "x" else ys[:, None]) * np.ones_like(U[0])
    speed = e.cp if wave == "P" else e.cs
    f = _pulse(pos - (LEN / 2 - TRAVEL / 2) - speed * t)
    ratio = c["lam"] / (c["lam"] + 2.0 * c["G"])
    for side in (0, 11):
        if wave == "P":
            d = 0 if along == "x" else 1           # vx / vy
            sdd = 3 if along == "x" else 4         # sxx / syy
            other = (4, 5) if along == "x" else (3, 5)
            U[side + sdd] += f
            U[side + d] += -f / c["Zp"]
            for o in other:
                U[side + o] += ratio * f
        else:                                       # S wave polarised across the direction, in-plane
            d = 1 if along == "x" else 0           # vy / vx
            U[side + 6] += f                       # sxy
            U[side + d] += -f / c["Zs"]
    return U


def _error(n: int, along: str, wave: str) -> float:
    sc = _scenario(n, along, wave)
    U = _wave_state(sc, along, wave, 0.0)
    dt = sc.dt()
    speed = sc.elastic.cp if wave == "P" else sc.elastic.cs
    steps = int(math.ceil(TRAVEL / (speed * dt)))
    dt = TRAVEL / (speed * steps)
    boxes = [(0, 0, sc.nx - 1, sc.ny - 1)]
    t = 0.0
    for _ in range(steps):
        assert O.level_step(sc, U, None, boxes, t, dt, nthreads=4) == 0
        t += dt
    exact = _wave_state(sc, along, wave, t)
    comp = (3 if along == "x" else 4) if wave == "P" else 6
    if along == "x":
        j = G + sc.ny // 2
        got, ref = U[comp, j, G:-G], exact[comp, j, G:-G]
    else:
        i = G + sc.nx // 2
        got, ref = U[comp, G:-G, i], exact[comp, G:-G, i]
    return float(np.sum(np.abs(got - ref)) * sc.dx / (AMP * WIDTH))


@pytest.mark.parametrize("along,wave", [("x", "P"), ("y", "P"), ("x", "S"), ("y", "S")])
def test_plane_wave_converges_at_second_order(along, wave):
    errs = [_error(n, along, wave) for n in (64, 128, 256)]
    orders = [math.log2(errs[k] / errs[k + 1]) for k in range(2)]
    print(f"{wave} along {along}: L1 errors {['%.2e' % e for e in errs]}, orders {['%.2f' % o for o in orders]}")
    assert errs[2] < 2e-3
    assert orders[1] > 1.6


def uniform_sliding_scenario(prec=A.TMK_PREC_FP64):
    """A slip-weakening fault loaded above its static strength everywhere
    (tau0 = 81.6 MPa > mu_s sigma_n = 81.24 MPa, no nucleation patch) with an
    instant weakening (Dc = 1e-9 m): every face slides from the first step."""
    sc = S.slip_weakening(nx=64, ny=32, dx=0.1, precision=prec)
    sc.sw.num_patches = 0
    sc.sw.dw = 1e-9
    sc.elastic.sxy0 = 81.6
    return sc


def uniform_sliding_answer(sc):
    """Exact answer of the 1-D problem the uniform fault poses: shear waves carry
    the stress drop away at either side, so the traction sits at the dynamic
    strength mu_d sigma_n and the slip rate is V = 2 (tau0 - mu_d sigma_n) / Zs."""
    c = sc.constants()
    sn = -sc.elastic.syy0
    return 2.0 * (sc.elastic.sxy0 - sc.sw.fd * sn) / c["Zs"], sc.sw.fd * sn


def test_uniformly_sliding_fault_radiates_at_the_exact_slip_rate():
    """Slip-weakening boundary data after 12 steps on the faces away from the
    domain's x edges: slip rate (component 4, and its x part 0), traction (2) and
    slip (5, 7) equal the exact answer to rounding; the cells next to the fault
    carry the dynamic shear stress to within 1 % of the stress drop (the
    scheme's smearing of the stress front, which the first step's static
    strength also shapes)."""
    sc = uniform_sliding_scenario()
    V, tau_d = uniform_sliding_answer(sc)
    U, B = sc.initial_U(), sc.initial_B()
    dt = sc.dt()
    t = 0.0
    for _ in range(12):
        assert O.level_step(sc, U, B, [(0, 0, sc.nx - 1, sc.ny - 1)], t, dt) == 0
        t += dt
    mid = slice(G + 24, G + 40)               # faces beyond the x edges' reach (cp t < 1.1 km)
    np.testing.assert_allclose(B[4, mid], V, rtol=1e-12)
    np.testing.assert_allclose(B[0, mid], V, rtol=1e-12)
    np.testing.assert_allclose(B[2, mid], tau_d, rtol=1e-12)
    np.testing.assert_allclose(B[5, mid], V * t, rtol=1e-12)
    np.testing.assert_allclose(B[7, mid], V * t, rtol=1e-12)
    np.testing.assert_allclose(U[6, G, mid], tau_d, atol=0.01 * (sc.elastic.sxy0 - tau_d))


def uniform_rs_scenario(prec=A.TMK_PREC_FP64):
    """A rate-and-state fault (aging law, velocity strengthening a=0.012,
    b=0.008, L=0.2 m, no nucleation) in steady sliding at 0.5 m/s whose shear
    load is then 2 MPa above that state's: every face speeds up and relaxes
    together, the 1-D problem of a uniformly sliding fault."""
    sc = S.rate_state(nx=128, ny=64, dx=0.05, precision=prec)
    rs = sc.rs
    rs.nsig = 0.0
    rs.a, rs.b, rs.L = 0.012, 0.008, 0.2
    sn = -sc.elastic.syy0
    Zs = sc.constants()["Zs"]
    Vi = 0.5
    rs.psi_init = rs.f0 - rs.b * math.log(Vi / rs.V0)            # aging-law steady state at Vi
    tau_f = sn * rs.a * math.asinh(Vi / (2 * rs.V0) * math.exp(rs.psi_init / rs.a))
    sc.elastic.sxy0 = tau_f + 0.5 * Zs * Vi + 2.0
    return sc


def uniform_rs_answer(sc, t_end):
    """The 1-D problem's exact evolution: the traction is tau0 - (Zs/2) V
    (radiation damping) = sn a asinh(V e^(psi/a) / (2 V0)), and the aging law
    d psi/dt = (b/L) (V0 e^(-(psi - f0)/b) - V), integrated to 1e-12.
    Returns (V(t), psi(t))."""
    from scipy.integrate import solve_ivp
    from scipy.optimize import brentq
    rs = sc.rs
    sn = -sc.elastic.syy0
    tau0 = sc.elastic.sxy0
    Zs = sc.constants()["Zs"]

    def V_of(psi):
        f = lambda V: tau0 - 0.5 * Zs * V - sn * rs.a * math.asinh(V / (2 * rs.V0) * math.exp(psi / rs.a))
        return brentq(f, 0.0, 2.0 * tau0 / Zs, xtol=1e-15, rtol=1e-15)

    def rhs(t, y):
        return [rs.b / rs.L * (rs.V0 * math.exp(-(y[0] - rs.f0) / rs.b) - V_of(y[0]))]

    sol = solve_ivp(rhs, (0.0, t_end), [rs.psi_init], rtol=1e-12, atol=1e-14, dense_output=True, method="DOP853")
    return (lambda t: V_of(float(sol.sol(t)[0]))), (lambda t: float(sol.sol(t)[0]))


def test_uniformly_sliding_rate_and_state_fault_follows_its_ode():
    """60 steps (until the domain's x edges' disturbances could reach the centre
    faces): the slip rate the level step stores (boundary component 2) is the
    ODE's at the step's midpoint, where the scheme's time-centred face state
    sits, to 1e-5, and the state variable (component 10) the ODE's at the step's
    end to 1e-6; the slip rate changes by 8 % over the run."""
    sc = uniform_rs_scenario()
    U, B = sc.initial_U(), sc.initial_B()
    dt = sc.dt()
    V_ode, psi_ode = uniform_rs_answer(sc, 61 * dt)
    c = G + sc.nx // 2
    t = 0.0
    Vs = []
    for _ in range(60):
        assert O.level_step(sc, U, B, [(0, 0, sc.nx - 1, sc.ny - 1)], t, dt) == 0
        t += dt
        V = V_ode(t - 0.5 * dt)
        assert abs(B[2, c] - V) <= 1e-5 * V, (t, B[2, c], V)
        assert abs(B[10, c] - psi_ode(t)) <= 1e-6, (t, B[10, c], psi_ode(t))
        np.testing.assert_allclose(B[2, c - 4:c + 4], B[2, c], rtol=1e-7)      # uniform along the fault
        Vs.append(B[2, c])
    assert Vs[-1] / Vs[0] > 1.05
