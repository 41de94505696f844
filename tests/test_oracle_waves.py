"""Known answers of the elastic wave equation for the oracle's level step.

A smooth plane P wave travelling along x and a plane S wave travelling along y
(no fault, absorbing edges) are advanced by the oracle's LinElastLevelGodunov
step and compared with the exact solution, the initial pulse translated by the
wave speed: the error must fall at close to second order as the grid is
refined (PPM with primitive limiting, corner transport upwind).  The comparison
row (column) lies outside the region the domain edges reach in the time run.
Oblique plane waves, in 2-D and in 3-D (the CH_SPACEDIM == 3 step), add the
transverse corrections, which an axis-aligned wave leaves at zero.  Two fault
problems with a 1-D exact answer close the set: a uniformly sliding
slip-weakening fault and a uniformly sliding rate-and-state fault.
The plain FP64 GPU form equals the oracle step for step (test_gpu_march.py,
test_gpu_parity.py, test_gpu_3d.py), so these answers pin it as well.

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
    boxes = O.tile_boxes(sc.nx, sc.ny, 64)    # patches for the oracle's threads; the exchange makes them one
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


# A P pulse meeting the x-hi domain edge head-on: a free surface (zero
# traction) reflects it with the stress reversed, sigma_xx = f(x - ct) -
# f(2X - x - ct), v_x = -(f(x - ct) + f(2X - x - ct)) / Zp (no mode conversion
# at normal incidence); an absorbing edge lets it leave, sigma_xx =
# f(x - ct).  The pulse starts 1.5 km from the edge and travels 3 km; the
# side edges are 4.5 km from the compared row (beyond cp t + the stencil's
# spread).
EDGE_TRAVEL = 3.0      # km
EDGE_SIDE = 9.0        # km


def edge_scenario(n: int, free: bool):
    """No background shear: a free surface would release it as an S wave."""
    dx = LEN / n
    e = S._elastic()
    e.sxy0 = 0.0
    return S.Scenario(name="edge_wave", nx=n, ny=int(round(EDGE_SIDE / dx)), dx=dx, cfl=0.9, elastic=e,
                      scheme=S._scheme(A.TMK_FAULT_NONE, bc=(0, 1 if free else 0, 0, 0, 0, 0)))


def edge_state(sc, free: bool, t: float) -> np.ndarray:
    c = sc.constants()
    U = sc.initial_U()
    xs = (np.arange(sc.nx + 2 * G) - G + 0.5) * sc.dx
    X = xs[None, :] * np.ones_like(U[0])
    x0 = LEN - EDGE_TRAVEL / 2
    f_in = _pulse(X - x0 - sc.elastic.cp * t)
    f_re = -_pulse(2 * LEN - X - x0 - sc.elastic.cp * t) if free else 0.0 * X
    r = c["lam"] / (c["lam"] + 2.0 * c["G"])
    for side in (0, 11):
        U[side + 3] += f_in + f_re
        U[side + 0] += (-f_in + f_re) / c["Zp"]
        U[side + 4] += r * (f_in + f_re)
        U[side + 5] += r * (f_in + f_re)
    return U


@pytest.mark.parametrize("free", [True, False], ids=["free_surface", "absorbing"])
def test_pulse_at_a_domain_edge_converges_at_second_order(free):
    """vx, sxx, syy along the middle row converge to the reflected (free
    surface) or departed (absorbing) pulse at order 1.9-2.5 from 64 to 256
    cells; there syy - r sxx, the zero-speed characteristic of x, stays as it
    was to rounding."""
    errs = []
    for n in (64, 128, 256):
        sc = edge_scenario(n, free)
        U = edge_state(sc, free, 0.0)
        c = sc.constants()
        r = c["lam"] / (c["lam"] + 2.0 * c["G"])
        w0 = U[4] - r * U[3]
        steps = int(math.ceil(EDGE_TRAVEL / (sc.elastic.cp * sc.dt())))
        dt = EDGE_TRAVEL / (sc.elastic.cp * steps)
        for k in range(steps):
            assert O.level_step(sc, U, None, O.tile_boxes(sc.nx, sc.ny, 64), k * dt, dt, nthreads=4) == 0
        exact = edge_state(sc, free, steps * dt)
        j = G + sc.ny // 2
        errs.append(np.array([np.sum(np.abs(U[q, j, G:-G] - exact[q, j, G:-G])) * sc.dx / (AMP * WIDTH)
                              for q in (0, 3, 4)]))
        assert np.max(np.abs((U[4] - r * U[3] - w0)[j, G:-G])) < 1e-12
    orders = np.log2(errs[1] / errs[2])
    print(f"{'free surface' if free else 'absorbing'}: errors at 256 {errs[2]}, orders {orders}")
    assert np.all(errs[2] < 2e-3)
    assert np.all(orders > 1.8)


# An antiplane (SH) pulse reflected by the free surface at x-hi: no mode
# conversion, the reflected pulse mirrors the incident one with the same
# amplitude, so sigma_xz vanishes and v_z doubles at the wall.  Compared in the
# strip within 2.5 km of the wall and 1 km of the centre line.
def sh_reflection_errors(theta_deg: float, ns=(64, 128, 256)):
    L, d0, travel = 11.0, 1.2, 2.4
    th = math.radians(theta_deg)
    n0, n1 = math.cos(th), math.sin(th)
    out = []
    for n in ns:
        e = S._elastic()
        e.sxy0 = 0.0
        sc = S.Scenario(name="sh_reflection", nx=n, ny=n, dx=L / n, cfl=0.9, elastic=e,
                        scheme=S._scheme(A.TMK_FAULT_NONE, bc=(0, 1, 0, 0, 0, 0)))
        x, y = _centres(sc, (0, 0, n - 1, n - 1), sc.dx, G)

        def state(t):
            cs, X = sc.elastic.cs, 0.5 * L
            f = _pulse(x * n0 + y * n1 - (X * n0 - d0) - cs * t)
            g = _pulse(-x * n0 + y * n1 + X * n0 + d0 - cs * t)       # the mirror image in x = X
            U = np.empty((22,) + x.shape)
            U[:] = sc.background()[:, None, None]
            for side in (0, 11):
                U[side + 2] += -(f + g) / sc.constants()["Zs"]
                U[side + 7] += (f - g) * n0
                U[side + 8] += (f + g) * n1
            return U

        U = state(0.0)
        steps = int(math.ceil(travel / (sc.elastic.cs * sc.dt())))
        dt = travel / (sc.elastic.cs * steps)
        for k in range(steps):
            assert O.level_step(sc, U, None, O.tile_boxes(n, n, 32), k * dt, dt, nthreads=4) == 0
        exact = state(steps * dt)
        strip = (x > 0.5 * L - 2.5) & (np.abs(y) < 1.0)
        out.append(np.array([np.sum(np.abs(U[q] - exact[q])[strip]) * sc.dx ** 2 / (AMP * WIDTH) for q in (2, 7, 8)]))
    return np.array(out)


def test_sh_pulse_reflected_by_a_free_surface():
    """Normal incidence: v_z and sigma_xz converge at second order (64 -> 256
    cells).  At 30 degrees sigma_xz still converges at second order, and v_z
    and sigma_yz at least at first order (the scheme's edge cells take
    one-sided differences)."""
    e0 = sh_reflection_errors(0.0)
    o0 = np.log2(e0[1, :2] / e0[2, :2])
    assert np.all(o0 > 1.8), o0
    e30 = sh_reflection_errors(30.0)
    o30 = np.log2(e30[1] / e30[2])
    assert o30[1] > 1.8 and o30[0] > 0.9 and o30[2] > 0.9, o30
    assert np.all(e30[2] < 0.1)


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


@pytest.mark.parametrize("r", [2, 4])
def test_uniformly_sliding_fault_through_amr(r):
    """The uniformly sliding slip-weakening fault (instant weakening) under a
    subcycled two-level hierarchy whose fine level covers the fault row from
    x = 0.8 to 5.6 km (rows 0-7 of the coarse grid): after 10 coarse steps the
    fine faces at the box's centre and the coarse faces there (the fine fault
    data averaged down) carry the exact slip rate, traction and slip to
    rounding.  (Within cp t of the fine box's x edges the coarse state's linear
    interpolation in time across the radiated front moves V by a few percent.)"""
    sc = uniform_sliding_scenario()          # 64 x 32 cells of 0.1 km
    V, tau_d = uniform_sliding_answer(sc)
    nb = sc.nbdry
    levels = []
    for dom, dx, boxes in (((0, 0, 63, 31), sc.dx, O.tile_boxes(64, 32, 16)),
                           ((0, 0, 64 * r - 1, 32 * r - 1), sc.dx / r, [(8 * r, 0, 56 * r - 1, 8 * r - 1)])):
        lv = O.LevelData(dom, dx, boxes, nb)
        for p, b in enumerate(lv.boxes):
            lv.U[p][:] = sc.background()[:, None, None]
            if lv.B[p] is not None:
                lv.B[p][:] = sc.initial_B(xlo=b[0], xhi=b[2])
        levels.append(lv)
    dt = sc.dt()
    assert O.amr_run(sc, levels, [r], 0.0, dt, 10, nthreads=4) == 0
    t = 10 * dt
    C, F = levels
    fine = F.B[0][:, G:-G][:, 24 * r - 4 * r:24 * r + 4 * r]        # fine faces of coarse x 28..35
    coarse = np.concatenate([C.B[p][:, G:-G] for p in range(len(C.boxes)) if C.B[p] is not None], axis=1)[:, 28:36]
    for B in (fine, coarse):
        np.testing.assert_allclose(B[4], V, rtol=1e-13)
        np.testing.assert_allclose(B[2], tau_d, rtol=1e-13)
        np.testing.assert_allclose(B[7], V * t, rtol=1e-13)


def test_uniformly_sliding_fault_with_linear_weakening():
    """Slip weakening over Dc = 0.4 m (ibcLinElast/SWIBCF.ChF:208, f = fs -
    (fs - fd) slip / Dc) on the uniformly loaded fault: while slip D < Dc the
    1-D problem gives D' = a + b D, a = 2 (tau0 - fs sn) / Zs, b = 2 (fs - fd)
    sn / (Zs Dc), so V = a e^(bt) and D = (a/b)(e^(bt) - 1).  After 0.36 s (24,
    48, 96 steps of dt, dt/2, dt/4) the slip rate converges at first order
    (friction takes the slip of the step before) and the slip at second
    order; the state stays uniform along the fault."""
    def scenario():
        sc = S.slip_weakening(nx=128, ny=32, dx=0.1)
        sc.sw.num_patches = 0
        sc.sw.dw = 0.4
        sc.elastic.sxy0 = 81.6
        return sc
    sc = scenario()
    Zs, sn = sc.constants()["Zs"], -sc.elastic.syy0
    a = 2.0 * (sc.elastic.sxy0 - sc.sw.fs * sn) / Zs
    b = 2.0 * (sc.sw.fs - sc.sw.fd) * sn / (Zs * sc.sw.dw)
    T = 24 * sc.dt()
    V_ex, D_ex = a * math.exp(b * T), a / b * (math.exp(b * T) - 1.0)
    assert D_ex < sc.sw.dw
    errs = []
    for k in (1, 2, 4):
        sc = scenario()
        U, B = sc.initial_U(), sc.initial_B()
        dt = sc.dt() / k
        for n in range(24 * k):
            assert O.level_step(sc, U, B, O.tile_boxes(sc.nx, sc.ny, 64), n * dt, dt, nthreads=4) == 0
        c = G + sc.nx // 2
        errs.append([B[4, c] / V_ex - 1.0, B[7, c] / D_ex - 1.0])
        assert np.ptp(B[4, c - 8:c + 8]) == 0.0
    errs = np.array(errs)
    orders = np.log2(np.abs(errs[:-1] / errs[1:]))
    print("linear weakening: errors (V, D)", errs.tolist(), "orders", orders.tolist())
    assert np.all((orders[:, 0] > 0.9) & (orders[:, 0] < 1.2))
    assert np.all((orders[:, 1] > 1.8) & (orders[:, 1] < 2.1))
    assert abs(errs[-1, 0]) < 0.03 and abs(errs[-1, 1]) < 1e-3


def uniform_rs_scenario(prec=A.TMK_PREC_FP64, law=A.TMK_RS_AGING_LAW, ab=(0.012, 0.008)):
    """A rate-and-state fault (aging law, or the reference's slip law;
    velocity strengthening a=0.012, b=0.008 by default, or weakening with
    the benchmarked a=0.008, b=0.012; L=0.2 m, no nucleation) in steady
    sliding at 0.5 m/s whose shear load is then 2 MPa above that state's:
    every face speeds up together, the 1-D problem of a uniformly sliding
    fault.  Both laws share the steady state."""
    sc = S.rate_state(nx=128, ny=64, dx=0.05, precision=prec, state_law=law)
    rs = sc.rs
    rs.nsig = 0.0
    rs.a, rs.b = ab
    rs.L = 0.2
    sn = -sc.elastic.syy0
    Zs = sc.constants()["Zs"]
    Vi = 0.5
    rs.psi_init = rs.f0 - rs.b * math.log(Vi / rs.V0)            # aging-law steady state at Vi
    tau_f = sn * rs.a * math.asinh(Vi / (2 * rs.V0) * math.exp(rs.psi_init / rs.a))
    sc.elastic.sxy0 = tau_f + 0.5 * Zs * Vi + 2.0
    return sc


def uniform_rs_answer(sc, t_end):
    """The 1-D problem's exact evolution: the traction is tau0 - (Zs/2) V
    (radiation damping) = sn a asinh(V e^(psi/a) / (2 V0)) = sn f, and the
    aging law d psi/dt = (b/L) (V0 e^(-(psi - f0)/b) - V) or the slip law
    d psi/dt = -(V/L) (f - f0 + (b - a) ln(V/V0)), integrated to 1e-12.
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
        V = V_of(y[0])
        if rs.state_law == A.TMK_RS_SLIP_LAW:
            f = rs.a * math.asinh(V / (2 * rs.V0) * math.exp(y[0] / rs.a))
            return [-(V / rs.L) * (f - rs.f0 + (rs.b - rs.a) * math.log(V / rs.V0))]
        return [rs.b / rs.L * (rs.V0 * math.exp(-(y[0] - rs.f0) / rs.b) - V)]

    sol = solve_ivp(rhs, (0.0, t_end), [rs.psi_init], rtol=1e-12, atol=1e-14, dense_output=True, method="DOP853")
    return (lambda t: V_of(float(sol.sol(t)[0]))), (lambda t: float(sol.sol(t)[0]))


@pytest.mark.parametrize("ab", [(0.012, 0.008), (0.008, 0.012)], ids=["strengthening", "weakening"])
def test_uniformly_sliding_rate_and_state_fault_follows_its_ode(ab):
    """60 steps (until the domain's x edges' disturbances could reach the centre
    faces): the slip rate the level step stores (boundary component 2) is the
    ODE's at the step's midpoint, where the scheme's time-centred face state
    sits, to 1e-5, and the state variable (component 10) the ODE's at the step's
    end to 1e-6; the slip rate grows by over 5 % in the run."""
    sc = uniform_rs_scenario(ab=ab)
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


def slip_law_errors(level_steps, ks=(1, 2, 4), nbase: int = 40):
    """The slip-law fault of uniform_rs_scenario stepped nbase * k times by
    dt / k with level_steps(sc, U, B, n, dt) (the state updated in place):
    per k, the relative error of the slip rate (component 2) against the ODE
    at the last step's midpoint and the error of the state (10) at its end."""
    out = []
    for k in ks:
        sc = uniform_rs_scenario(law=A.TMK_RS_SLIP_LAW)
        U, B = sc.initial_U(), sc.initial_B()
        dt = sc.dt() / k
        n = nbase * k
        V_ode, psi_ode = uniform_rs_answer(sc, (n + 1) * dt)
        level_steps(sc, U, B, n, dt)
        c = G + sc.nx // 2
        t = n * dt
        out.append((B[2, c] / V_ode(t - 0.5 * dt) - 1.0, B[10, c] - psi_ode(t)))
    return np.array(out)


def test_uniformly_sliding_slip_law_fault_converges_at_first_order():
    """The reference's slip law (ibcLinElast/RSIBCF.ChF:127-132) advances the
    state by one explicit step psi -= dt (V/L)(f - fss): the uniformly sliding
    fault reaches its ODE at first order in dt (40, 80, 160 steps of dt, dt/2,
    dt/4 over the same time: slip-rate and state errors halve with dt)."""
    def steps(sc, U, B, n, dt):
        for k in range(n):
            assert O.level_step(sc, U, B, O.tile_boxes(sc.nx, sc.ny, 64), k * dt, dt, nthreads=4) == 0
    e = slip_law_errors(steps)
    orders = np.log2(np.abs(e[:-1] / e[1:]))
    print("slip law: errors (V, psi)", e.tolist(), "orders", orders.tolist())
    assert np.all(np.abs(orders - 1.0) < 0.1)
    assert abs(e[-1, 0]) < 2e-4 and abs(e[-1, 1]) < 1e-5


# Viscoplastic relaxation (srcLinElast/PlasticPhysicsF.ChF:74-181): a uniform
# state above the Drucker-Prager yield surface feels no flux, so each level
# step changes it only by the plastic correction, whose lambda =
# Y / (dt (h + G + mu beta K) + eta) makes it one backward-Euler step of
# dY/dt = -k Y / eta, k = G + mu beta K + h: after n steps the overstress is
# exactly Y0 (eta / (eta + k dt))^n and the plastic strain (Y0 - Y) / k.
def plastic_scenario(h: float = 0.0):
    """No fault, absorbing edges, the 120 MPa / 70 MPa background (Y0 = 71 MPa
    above yield) with the decks' Drucker-Prager parameters and hardening h."""
    sc = S.Scenario(name="plastic_relaxation", nx=64, ny=64, dx=0.1, cfl=0.9, elastic=S._elastic(),
                    scheme=S._scheme(A.TMK_FAULT_NONE, plasticity=1, bc=(0, 0, 0, 0, 0, 0)),
                    plastic=S.plastic_params())
    sc.plastic.h = h
    return sc


def overstress(sc, u) -> float:
    """Y = sqrt(J2) - max(b + h gamma - mu sigma_mean, 0) of one side's cell state u (11 comps)."""
    p = sc.plastic
    sxx, syy, szz, sxy, sxz, syz = u[3:9]
    sig = (sxx + syy + szz) / 3.0
    J2 = ((sxx - syy) ** 2 + (syy - szz) ** 2 + (szz - sxx) ** 2) / 6.0 + sxy ** 2 + sxz ** 2 + syz ** 2
    return math.sqrt(J2) - max(-p.mu * sig + p.b + u[10] * p.h, 0.0)


def plastic_k(sc) -> float:
    c = sc.constants()
    return c["G"] + sc.plastic.mu * sc.plastic.beta * (c["lam"] + 2.0 * c["G"] / 3.0) + sc.plastic.h


@pytest.mark.parametrize("h", [0.0, 5.0], ids=["no_hardening", "hardening"])
def test_viscoplastic_relaxation_of_a_uniform_state(h):
    """16 level steps at the CFL step: the centre cell's overstress equals the
    backward-Euler closed form to 1e-12 of Y0 and its plastic strain (Y0 - Y)/k
    to rounding, both sides, the state uniform around it.  Over two relaxation
    times eta/k with 4, 8, 16, 32 steps the overstress reaches the ODE's
    Y0 exp(-k t / eta) at first order (orders within 0.15 of 1)."""
    sc = plastic_scenario(h)
    k = plastic_k(sc)
    eta = sc.plastic.eta
    U = sc.initial_U()
    c = G + 32
    Y0 = overstress(sc, U[:11, c, c])
    assert Y0 > 50.0
    dt = sc.dt()
    for n in range(16):
        assert O.level_step(sc, U, None, O.tile_boxes(64, 64, 32), n * dt, dt, nthreads=4) == 0
    Yd = Y0 * (eta / (eta + k * dt)) ** 16
    for side in (0, 11):
        u = U[side:side + 11, c, c]
        assert abs(overstress(sc, u) - Yd) <= 1e-12 * Y0
        assert abs(u[10] - (Y0 - Yd) / k) <= 1e-14 * Y0 / k
    assert np.ptp(U[3:9, c - 4:c + 4, c - 4:c + 4], axis=(1, 2)).max() == 0.0

    T = 2.0 * eta / k
    errs = []
    for n in (4, 8, 16, 32):
        sc = plastic_scenario(h)
        U = sc.initial_U()
        dt = T / n
        assert dt <= sc.dt()
        for s in range(n):
            assert O.level_step(sc, U, None, O.tile_boxes(64, 64, 32), s * dt, dt, nthreads=4) == 0
        errs.append(overstress(sc, U[:11, c, c]) / (Y0 * math.exp(-k * T / eta)) - 1.0)
    orders = np.log2(np.array(errs[:-1]) / np.array(errs[1:]))
    print(f"plastic relaxation h={h}: ODE errors {errs}, orders {orders}")
    assert np.all(np.abs(orders - 1.0) < 0.15)


# Oblique plane waves: the pulse travels along n = (cos th, sin th), so every
# direction's transverse correction of the corner transport upwind scheme
# carries it (an axis-aligned wave has zero transverse differences).  The
# square domain's edges send waves inward from the first step; the error is
# measured on the central disc of radius R, which they do not reach in the
# pulse's travel time (cp t + R + stencil spread below the half-width).
OBLIQUE_TH = math.radians(30.0)
OBLIQUE_R = 1.5                       # km
OBLIQUE_LEN = {"P": 8.0, "S": 11.0, "SH": 11.0}   # km, side of the square domain


def oblique_scenario(n: int, wave: str):
    return S.Scenario(name="oblique_wave", nx=n, ny=n, dx=OBLIQUE_LEN[wave] / n, cfl=0.9,
                      elastic=S._elastic(), scheme=S._scheme(A.TMK_FAULT_NONE, bc=(0, 0, 0, 0, 0, 0)))


def wave_at(sc, wave: str, x: np.ndarray, y: np.ndarray, t: float) -> np.ndarray:
    """The oblique wave at time t at cell centres (x, y), measured from the
    domain's centre, on the scenario's background.  A P wave along n carries
    v = -f/Zp n, sigma = f (r I + (1 - r) n n^T), r = lam/(lam + 2G); an S wave
    polarised in-plane along m = (-n_y, n_x) carries v = -f/Zs m,
    sigma = f (n m^T + m n^T); the antiplane (SH) wave, polarised along z,
    carries v_z = -f/Zs, sigma_xz = f n_x, sigma_yz = f n_y."""
    c = sc.constants()
    n = (math.cos(OBLIQUE_TH), math.sin(OBLIQUE_TH))
    m = (-n[1], n[0])
    speed = sc.elastic.cp if wave == "P" else sc.elastic.cs
    f = _pulse(x * n[0] + y * n[1] + 0.5 * TRAVEL - speed * t)
    r = c["lam"] / (c["lam"] + 2.0 * c["G"])
    U = np.empty((22,) + x.shape)
    U[:] = sc.background()[:, None, None]
    for side in (0, 11):
        if wave == "P":
            for d in range(2):
                U[side + d] += -f / c["Zp"] * n[d]
                U[side + 3 + d] += f * (r + (1.0 - r) * n[d] * n[d])
            U[side + 5] += r * f
            U[side + 6] += f * (1.0 - r) * n[0] * n[1]
        elif wave == "S":
            for d in range(2):
                U[side + d] += -f / c["Zs"] * m[d]
                U[side + 3 + d] += 2.0 * f * n[d] * m[d]
            U[side + 6] += f * (n[0] * m[1] + n[1] * m[0])
        else:
            U[side + 2] += -f / c["Zs"]
            U[side + 7] += f * n[0]
            U[side + 8] += f * n[1]
    return U


def _centres(sc, b, dx: float, ghost: int):
    """Cell-centre coordinates, from the domain's centre, of box b grown by
    `ghost` cells on a level of cell size dx."""
    yy, xx = np.mgrid[b[1] - ghost:b[3] + ghost + 1, b[0] - ghost:b[2] + ghost + 1]
    return (xx + 0.5) * dx - 0.5 * sc.nx * sc.dx, (yy + 0.5) * dx - 0.5 * sc.ny * sc.dx


def oblique_state(sc, wave: str, t: float):
    """(U, r2): the state of the whole level at time t, ghosts included, and
    the squared distance of each cell centre from the domain's centre."""
    x, y = _centres(sc, (0, 0, sc.nx - 1, sc.ny - 1), sc.dx, G)
    return wave_at(sc, wave, x, y, t), x * x + y * y


# the components each wave carries: vx, vy, sxx, syy, sxy (in-plane); vz, sxz, syz (antiplane)
OBLIQUE_COMPS = {"P": (0, 1, 3, 4, 6), "S": (0, 1, 3, 4, 6), "SH": (2, 7, 8)}


def oblique_steps(sc, wave: str):
    speed = sc.elastic.cp if wave == "P" else sc.elastic.cs
    steps = int(math.ceil(TRAVEL / (speed * sc.dt())))
    return steps, TRAVEL / (speed * steps)


def oblique_error(sc, wave: str, U: np.ndarray, t: float) -> np.ndarray:
    """L1 error over the central disc per component the wave carries,
    normalised by the pulse's amplitude and width."""
    exact, r2 = oblique_state(sc, wave, t)
    disc = r2 <= OBLIQUE_R ** 2
    return np.array([np.sum(np.abs(U[c] - exact[c])[disc]) * sc.dx ** 2 / (AMP * WIDTH)
                     for c in OBLIQUE_COMPS[wave]])


@pytest.mark.parametrize("wave", ["P", "S", "SH"])
def test_oblique_plane_wave_converges_at_second_order(wave):
    """Every component's error falls at order 2.0-2.1 from 64 to 256 cells a
    side (the level tiled into 32x32 patches, which the exchange makes
    equivalent to one patch)."""
    errs = []
    for n in (64, 128, 256):
        sc = oblique_scenario(n, wave)
        U, _ = oblique_state(sc, wave, 0.0)
        steps, dt = oblique_steps(sc, wave)
        t = 0.0
        for _ in range(steps):
            assert O.level_step(sc, U, None, O.tile_boxes(n, n, 32), t, dt, nthreads=4) == 0
            t += dt
        errs.append(oblique_error(sc, wave, U, t))
    orders = np.log2(errs[1] / errs[2])
    print(f"oblique {wave}: errors at 256 {errs[2]}, orders 64->128 {np.log2(errs[0] / errs[1])}, 128->256 {orders}")
    assert np.all(errs[2] < 4e-3)
    assert np.all(orders > 1.8)


@pytest.mark.parametrize("wave", ["P", "SH"])
@pytest.mark.parametrize("order,charlim,expect", [(1, 0, (1.8, 2.2)), (0, 0, (0.85, 1.1)), (2, 1, (1.8, 2.2))],
                         ids=["plm", "first_order", "ppm_char_limiting"])
def test_oblique_wave_with_the_other_normal_predictors(wave, order, charlim, expect):
    """The decks' other normal predictors (LinElastPatchGodunov::PLMNormalPred
    with fourth-order slopes, the piecewise-constant one of normal_pred_order
    0, and PPM limited in characteristic instead of primitive variables) on
    the oblique wave: PLM and characteristic limiting converge at second
    order, the piecewise-constant predictor at first order (64 -> 256 cells)."""
    errs = []
    for n in (64, 128, 256):
        sc = oblique_scenario(n, wave)
        sc.scheme.normal_pred_order = order
        if charlim:
            sc.scheme.use_prim_limiting, sc.scheme.use_char_limiting = 0, 1
        U, _ = oblique_state(sc, wave, 0.0)
        steps, dt = oblique_steps(sc, wave)
        for k in range(steps):
            assert O.level_step(sc, U, None, O.tile_boxes(n, n, 32), k * dt, dt, nthreads=4) == 0
        errs.append(oblique_error(sc, wave, U, steps * dt))
    orders = np.log2(errs[1] / errs[2])
    assert np.all((orders > expect[0]) & (orders < expect[1])), orders


# The same in 3-D (CH_SPACEDIM == 3): a plane wave along a direction with no
# zero component, so that all six transverse corrections of the 3-D corner
# transport upwind step carry it; the S wave is polarised along the unit
# vector of the z axis' part normal to n, so that all nine components carry a
# pulse.  Error on the central ball of radius 1 km; the S pulse travels 1 km
# (the edges' P waves must stay out of the ball for its travel time).
N3 = np.array([1.0, 0.7, 0.5]) / np.linalg.norm([1.0, 0.7, 0.5])
M3 = np.array([0.0, 0.0, 1.0]) - N3[2] * N3
M3 /= np.linalg.norm(M3)
OBLIQUE3_LEN = {"P": 7.0, "S": 6.5}      # km, side of the cube
OBLIQUE3_TRAVEL = {"P": 2.0, "S": 1.0}   # km
OBLIQUE3_R = 1.0                         # km
_SYM = {(0, 0): 3, (1, 1): 4, (2, 2): 5, (0, 1): 6, (0, 2): 7, (1, 2): 8}


def oblique3_scenario(n: int, wave: str):
    return S.Scenario(name="oblique_wave_3d", nx=n, ny=n, dx=OBLIQUE3_LEN[wave] / n, cfl=0.9,
                      elastic=S._elastic(), scheme=S._scheme(A.TMK_FAULT_NONE, bc=(0, 0, 0, 0, 0, 0)))


def oblique3_state(sc, wave: str, t: float):
    """(U (22, n+8, n+8, n+8), r2) at time t, as oblique_state in 3-D."""
    c = sc.constants()
    n = sc.nx
    U = np.empty((22,) + (n + 2 * G,) * 3)
    U[:] = sc.background()[:, None, None, None]
    xs = (np.arange(n + 2 * G) - G + 0.5) * sc.dx - 0.5 * n * sc.dx
    Z, Y, X = np.meshgrid(xs, xs, xs, indexing="ij")
    speed = sc.elastic.cp if wave == "P" else sc.elastic.cs
    f = _pulse(X * N3[0] + Y * N3[1] + Z * N3[2] + 0.5 * OBLIQUE3_TRAVEL[wave] - speed * t)
    r = c["lam"] / (c["lam"] + 2.0 * c["G"])
    for side in (0, 11):
        for d in range(3):
            U[side + d] += -f / c["Zp"] * N3[d] if wave == "P" else -f / c["Zs"] * M3[d]
        for (i, j), q in _SYM.items():
            if wave == "P":
                U[side + q] += f * ((r if i == j else 0.0) + (1.0 - r) * N3[i] * N3[j])
            else:
                U[side + q] += f * (N3[i] * M3[j] + M3[i] * N3[j])
    return U, X * X + Y * Y + Z * Z


def oblique3_steps(sc, wave: str):
    speed = sc.elastic.cp if wave == "P" else sc.elastic.cs
    dt = sc.dt() / math.sqrt(3.0)          # the 3-D CFL bound
    steps = int(math.ceil(OBLIQUE3_TRAVEL[wave] / (speed * dt)))
    return steps, OBLIQUE3_TRAVEL[wave] / (speed * steps)


def oblique3_error(sc, wave: str, U: np.ndarray, t: float) -> np.ndarray:
    exact, r2 = oblique3_state(sc, wave, t)
    ball = r2 <= OBLIQUE3_R ** 2
    return np.array([np.sum(np.abs(U[c] - exact[c])[ball]) * sc.dx ** 3 / (AMP * WIDTH) for c in range(9)])


def oracle_steps_3d(sc, U: np.ndarray, steps: int, dt: float, B: np.ndarray | None = None, ny: int | None = None,
                    t0: float = 0.0, nthreads: int = 8) -> None:
    """Advance the cube U (n cells in x and z, ny in y; B the fault data of the
    y-lo plane, or None) by the oracle's 3-D patch step, the domain tiled into
    2x2x2 patches (2x1x2 with a fault) stepped on threads (the oracle's calls
    release the interpreter lock), each patch's ghost cells and fault data
    refilled from the level between steps as an exchange does."""
    from concurrent.futures import ThreadPoolExecutor
    n = sc.nx
    ny = n if ny is None else ny
    h = n // 2
    ys = (0,) if B is not None else (0, h)
    hy = ny if B is not None else h
    boxes = [((x0, y0, z0), (x0 + h - 1, y0 + hy - 1, z0 + h - 1)) for z0 in (0, h) for y0 in ys for x0 in (0, h)]
    cut = lambda lo, hi, g: (slice(None),) + tuple(slice(lo[d] + G - g, hi[d] + G + g + 1) for d in (2, 1, 0))
    bcut = lambda lo, hi, g: (slice(None), slice(lo[2] + G - g, hi[2] + G + g + 1), slice(lo[0] + G - g, hi[0] + G + g + 1))

    def one(box, t):
        lo, hi = box
        sub = np.ascontiguousarray(U[cut(lo, hi, G)])
        bs = np.ascontiguousarray(B[bcut(lo, hi, G)]) if B is not None else None
        rc, _ = O.patch_update_state_3d(sc, sub, tuple(v - G for v in lo), lo, hi, (0, 0, 0), (n - 1, ny - 1, n - 1),
                                        bs, (lo[0] - G, lo[2] - G), sc.dx, t, dt)
        assert rc == 0
        return sub, bs

    with ThreadPoolExecutor(nthreads) as pool:
        for k in range(steps):
            out = list(pool.map(lambda b: one(b, t0 + k * dt), boxes))
            for (lo, hi), (sub, bs) in zip(boxes, out):
                U[cut(lo, hi, 0)] = sub[:, G:-G, G:-G, G:-G]
                if bs is not None:
                    B[bcut(lo, hi, 0)] = bs[:, G:-G, G:-G]


@pytest.mark.parametrize("wave", ["P", "S"])
def test_oblique_plane_wave_3d_converges_at_second_order(wave):
    """Every one of the nine components converges at order 1.8-2.2 from 48 to
    64 cells a side (the step ratio is 4/3: order = log(e48/e64) / log(4/3))."""
    errs = []
    for n in (48, 64):
        sc = oblique3_scenario(n, wave)
        U, _ = oblique3_state(sc, wave, 0.0)
        steps, dt = oblique3_steps(sc, wave)
        oracle_steps_3d(sc, U, steps, dt)
        errs.append(oblique3_error(sc, wave, U, steps * dt))
    orders = np.log(errs[0] / errs[1]) / math.log(64 / 48)
    print(f"3-D oblique {wave}: errors at 64 {errs[1]}, orders {orders}")
    assert np.all(errs[1] < 1e-2)
    assert np.all(orders > 1.6)


# Through a refined hierarchy: the 2-D oblique wave crosses the coarse-fine
# interface of a centred fine square (2 km a side) at ratios 2 and 4, subcycled
# (AMRLevelLinElast::advance order: the coarse step, r fine steps with the
# coarse-fine ghost fill interpolated in time, refluxing, average-down).  Its
# error converges at second order on the fine level and on the coarse cells
# around it that it does not cover (within 1.5 km of the centre), so the
# fill, the flux registers and the average-down carry the wave to the
# scheme's accuracy.
AMR_FINE_HALF = 1.0     # km


def amr_wave_hierarchy(nc: int, r: int, wave: str):
    """(sc, [coarse, fine] LevelData at t = 0, covered coarse cell range, steps, dt)."""
    sc = oblique_scenario(nc, wave)
    k = int(round(AMR_FINE_HALF / sc.dx))
    c0, c1 = nc // 2 - k, nc // 2 + k - 1
    fb = (c0 * r, c0 * r, (c1 + 1) * r - 1, (c1 + 1) * r - 1)
    fboxes = [(i0, j0, min(i0 + 31, fb[2]), min(j0 + 31, fb[3]))
              for j0 in range(fb[1], fb[3] + 1, 32) for i0 in range(fb[0], fb[2] + 1, 32)]
    levels = []
    for dom, dx, boxes in (((0, 0, nc - 1, nc - 1), sc.dx, O.tile_boxes(nc, nc, 32)),
                           ((0, 0, nc * r - 1, nc * r - 1), sc.dx / r, fboxes)):
        lv = O.LevelData(dom, dx, boxes, 0)
        for p, b in enumerate(boxes):
            lv.U[p][:] = wave_at(sc, wave, *_centres(sc, b, dx, G), 0.0)
        levels.append(lv)
    steps, dt = oblique_steps(sc, wave)
    return sc, levels, (c0, c1), steps, dt


def amr_wave_errors(sc, wave: str, levels, covered, t: float, R: float = 1.5):
    """L1 errors (per component the wave carries) of the fine level's valid
    cells and of the coarse level's uncovered cells within R of the centre."""
    C, F = levels
    out = []
    for lv, coarse in ((F, False), (C, True)):
        e = np.zeros(len(OBLIQUE_COMPS[wave]))
        for p, b in enumerate(lv.boxes):
            x, y = _centres(sc, b, lv.dx, 0)
            exact = wave_at(sc, wave, x, y, t)
            mask = np.ones(x.shape, dtype=bool)
            if coarse:
                ii = np.arange(b[0], b[2] + 1)[None, :]
                jj = np.arange(b[1], b[3] + 1)[:, None]
                cov = (ii >= covered[0]) & (ii <= covered[1]) & (jj >= covered[0]) & (jj <= covered[1])
                mask = (x * x + y * y <= R * R) & ~cov
            u = lv.U[p][:, G:-G, G:-G]
            e += [np.sum(np.abs(u[c] - exact[c])[mask]) * lv.dx ** 2 for c in OBLIQUE_COMPS[wave]]
        out.append(e / (AMP * WIDTH))
    return out


@pytest.mark.parametrize("wave", ["P", "S", "SH"])
@pytest.mark.parametrize("r", [2, 4])
def test_oblique_wave_through_amr_converges_at_second_order(wave, r):
    """Coarse grids of 32, 64 and 128 cells a side: fine-level and coarse-level
    errors fall at order 1.9-2.2 from 64 to 128 in every component."""
    errs = []
    for nc in (32, 64, 128):
        sc, levels, covered, steps, dt = amr_wave_hierarchy(nc, r, wave)
        assert O.amr_run(sc, levels, [r], 0.0, dt, steps, nthreads=4) == 0
        errs.append(amr_wave_errors(sc, wave, levels, covered, steps * dt))
    fine = np.log2(errs[1][0] / errs[2][0])
    coarse = np.log2(errs[1][1] / errs[2][1])
    print(f"AMR r={r} {wave}: fine errors {errs[2][0]} orders {fine}; coarse errors {errs[2][1]} orders {coarse}")
    assert np.all(errs[2][0] < 5e-3) and np.all(errs[2][1] < 5e-3)
    assert np.all(fine > 1.8) and np.all(coarse > 1.8)


# The two uniformly sliding faults in 3-D (the fault the y-lo plane, the state
# uniform in x and z): the 1-D answers hold on the fault faces the x and z
# edges' disturbances have not reached.  The 3-D step predicts the boundary
# data over dt/3 where the 2-D step uses dt/2, so these pin the 3-D fault path
# that the reduction of a z-uniform state to the 2-D step leaves out.
def uniform_fault_3d(sc, n: int, ny: int):
    """(U, B) of a 2-D scenario's initial state repeated along z on an n x ny x n
    cube, ghosts included."""
    sc.nx, sc.ny = n, ny
    U = np.ascontiguousarray(np.repeat(sc.initial_U()[:, None], n + 2 * G, axis=1))
    B = np.ascontiguousarray(np.repeat(sc.initial_B()[:, None], n + 2 * G, axis=1))
    return U, B


def test_uniformly_sliding_faults_3d():
    """Slip weakening, 12 steps on a 32x16x32 cube: slip rate (components 4 and
    0), traction (2) and slip (5, 7) equal the exact answer to rounding on the
    central 8x8 faces, 12 cells from the x and z edges (the scheme's reach in
    12 steps; a cell nearer, the edges' disturbance is 3e-10 of the slip rate).  Rate and state, 30 steps on a 48x16x48 cube: the
    slip rate (2) is the ODE's at each step's midpoint to 1e-6 and the state
    (10) the ODE's at the step's end to 1e-8."""
    sc = uniform_sliding_scenario()
    V, tau_d = uniform_sliding_answer(sc)
    U, B = uniform_fault_3d(sc, 32, 16)
    dt = sc.dt() / math.sqrt(3.0)
    oracle_steps_3d(sc, U, 12, dt, B, ny=16)
    mid = (slice(G + 12, G + 20), slice(G + 12, G + 20))
    for comp, want in ((4, V), (0, V), (2, tau_d), (5, V * 12 * dt), (7, V * 12 * dt)):
        np.testing.assert_allclose(B[(comp,) + mid], want, rtol=1e-12, err_msg=f"component {comp}")

    sc = uniform_rs_scenario()
    U, B = uniform_fault_3d(sc, 48, 16)
    dt = sc.dt() / math.sqrt(3.0)
    V_ode, psi_ode = uniform_rs_answer(sc, 31 * dt)
    c = G + 24
    for k in range(3):
        oracle_steps_3d(sc, U, 10, dt, B, ny=16, t0=10 * k * dt)
        t = 10 * (k + 1) * dt
        V = V_ode(t - 0.5 * dt)
        face = (slice(c - 3, c + 3), slice(c - 3, c + 3))
        assert np.max(np.abs(B[(2,) + face] - V)) <= 1e-6 * V, (t, B[2, c, c], V)
        assert np.max(np.abs(B[(10,) + face] - psi_ode(t))) <= 1e-8, (t, B[10, c, c], psi_ode(t))
