"""Known-answer tests of the CPU oracle against properties of the reference formulas.

The reference ships no tests or golden vectors; these properties follow from
the formulas it implements (srcLinElast/LinElastPhysicsF.ChF,
ibcLinElast/RSIBCF.ChF, srcLinElast/PlasticPhysicsF.ChF).
"""
import math

import numpy as np
import pytest

import oracle as O
from tetemoko_gb300 import _capi as A, scenarios as S


@pytest.fixture(scope="module")
def sc():
    return S.rate_state(nx=64, ny=32, dx=0.1)


def _state(rng, sc):
    w = sc.background().copy()
    for c in range(22):
        if c % 11 < 3:
            w[c] += rng.normal(0, 0.5)
        elif c % 11 < 9:
            w[c] += rng.normal(0, 5.0)
    return w


def test_constants_follow_linelastset(sc):
    k = O.constants(sc)
    G = 2.670 * 3.464 ** 2
    assert math.isclose(k["rho"], G / 3.464 ** 2, rel_tol=1e-15)
    assert math.isclose(k["lam"], 6.0 ** 2 * k["rho"] - 2 * G, rel_tol=1e-14)
    assert math.isclose(k["Zs"], k["rho"] * 3.464, rel_tol=1e-15)
    assert math.isclose(k["Zp"], k["rho"] * 6.0, rel_tol=1e-15)


@pytest.mark.parametrize("idir", [0, 1])
def test_char_synthesis_inverts_analysis(sc, idir):
    rng = np.random.default_rng(idir)
    for _ in range(20):
        w = _state(rng, sc)
        w[[9, 10, 20, 21]] = rng.normal(0, 1, 4)
        back = O.charsynthesis(sc, O.charanalysis(sc, w, idir), idir)
        assert np.allclose(back, w, rtol=1e-13, atol=1e-12)


@pytest.mark.parametrize("idir", [0, 1])
def test_riemann_of_equal_states_is_that_state(sc, idir):
    rng = np.random.default_rng(10 + idir)
    for _ in range(20):
        w = _state(rng, sc)
        g = O.riemann(sc, w, w, idir)
        assert np.allclose(g, w, rtol=1e-13, atol=1e-12)


@pytest.mark.parametrize("idir,lohi", [(0, -1), (0, 1), (1, 1)])
def test_free_surface_has_zero_traction(sc, idir, lohi):
    rng = np.random.default_rng(20)
    w = _state(rng, sc)
    g = O.edge_bc(sc, w, lohi, idir, outflow=False)
    trac = {0: [3, 6, 7], 1: [4, 8, 6]}[idir]     # sxx sxy sxz on x faces; syy syz sxy on y faces
    for s in (0, 11):
        assert np.allclose(g[[s + c for c in trac]], 0.0, atol=1e-12)


def test_absorbing_edge_returns_background_at_rest(sc):
    bg = sc.background()
    for idir, lohi in [(0, -1), (0, 1), (1, 1)]:
        g = O.edge_bc(sc, bg, lohi, idir, outflow=True)
        ev = [c for c in range(22) if c % 11 < 9 and c % 11 not in (3, 4, 5)]
        assert np.allclose(g[ev], bg[ev], atol=1e-12), (idir, lohi)


def test_absorbing_edge_is_transparent_to_an_outgoing_wave(sc):
    """At the x-lo edge a wave leaving the domain carries only the left-going
    characteristics (sxx + Zp vx, sxy + Zs vy); the edge state equals the interior."""
    k = O.constants(sc)
    w = sc.background().copy()
    a, b = 3.0, -2.0
    w[0] += a / k["Zp"]; w[3] += a        # changes sxx + Zp vx only
    w[1] += b / k["Zs"]; w[6] += b        # changes sxy + Zs vy only
    g = O.edge_bc(sc, w, -1, 0, outflow=True)
    for c in (0, 1, 3, 6):
        assert math.isclose(g[c], w[c], rel_tol=1e-12, abs_tol=1e-12)
    # outgoing characteristic preserved, incoming one equals the background's
    assert math.isclose(g[3] + k["Zp"] * g[0], w[3] + k["Zp"] * w[0], abs_tol=1e-11)
    assert math.isclose(g[3] - k["Zp"] * g[0], sc.background()[3], abs_tol=1e-11)
    assert math.isclose(g[6] + k["Zs"] * g[1], w[6] + k["Zs"] * w[1], abs_tol=1e-11)
    assert math.isclose(g[6] - k["Zs"] * g[1], sc.background()[6], abs_tol=1e-11)


def test_rs_newton_residual_and_bracket(sc):
    """Where the root lies in the reference's bracket (0, phi/Zs) Newton finds it."""
    rng = np.random.default_rng(5)
    k = O.constants(sc)
    n = converged = 0
    while n < 200:
        phi = rng.uniform(1.0, 150.0)
        psi = rng.uniform(0.3, 0.9)
        sn = rng.uniform(20.0, 150.0)
        a = rng.uniform(0.006, 0.02)
        beta = math.exp(psi / a) / (2.0 * sc.rs.V0)
        if sn * a * math.asinh(beta * phi / k["Zs"]) < 0.5 * phi:
            continue                     # root beyond the bracket: see the next test
        n += 1
        V, tau, it = O.rs_newton(sc, phi, psi, sn, a, rng.uniform(0, 20))
        assert 0.0 <= V <= phi / k["Zs"]
        assert math.isclose(tau, sn * a * math.asinh(beta * V), rel_tol=1e-15)
        if it > 100:
            # bisection cannot reach roots many decades below the bracket (V* ~ 1e-35 m/s
            # for a strongly healed state); the reference gives up after IMAX silently
            continue
        converged += 1
        g = sn * a * math.asinh(beta * V) + 0.5 * k["Zs"] * V - phi
        assert abs(g) <= 1e-8 * phi, (phi, psi, sn, a, V, g, it)
    assert converged >= 150


def test_rs_newton_root_outside_the_bracket_ends_at_its_edge(sc):
    """The bracket (0, phi/Zs) of ibcLinElast/RSIBCF.ChF:358 excludes the root when
    sn a asinh(beta phi/Zs) < phi/2 (the damping term is Zs/2 V).  The reference then
    runs all IMAX = 100 iterations and returns the bracket edge; so does the oracle."""
    k = O.constants(sc)
    phi, psi, sn, a = 58.121963237042216, 0.5450839232519993, 25.88577520731787, 0.006682607950180353
    V, tau, it = O.rs_newton(sc, phi, psi, sn, a, 1.0)
    assert it == 101
    assert math.isclose(V, phi / k["Zs"], rel_tol=1e-12)


def test_rs_fault_at_steady_state_slides_at_the_initial_rate(sc):
    """With psi set for V = 1e-12 m/s at tau = 70, sn = 120 the locked fault slides at that rate."""
    w = sc.background()
    far = 40.0   # far from the nucleation Gaussian
    g = O.rs_fault(sc, w, sc.rs.psi_init, far)
    V = g[0] - g[11]
    assert math.isclose(V, 1e-12, rel_tol=1e-6)
    assert math.isclose(g[6], 70.0, rel_tol=1e-12)


def test_sw_fault_locked_below_strength():
    sc = S.slip_weakening(nx=64, ny=32, dx=0.1)
    w = sc.background()
    b = sc.initial_B(xlo=0, xhi=0)[:, 4]
    g = O.sw_fault(sc, w, b, xcell=0.05)      # far from the nucleation patch: tau 70 < 0.677*120
    assert abs(g[0] - g[11]) < 1e-12
    assert math.isclose(g[6], 70.0, rel_tol=1e-12)


def test_plastic_return_lands_on_yield_surface_without_viscosity():
    sc = S.slip_weakening(nx=8, ny=8, dx=0.1, plasticity=True)
    sc.plastic.eta = 0.0
    rng = np.random.default_rng(3)
    mu = sc.plastic.mu
    for _ in range(50):
        s = np.array([rng.uniform(-150, -50), rng.uniform(-150, -50), rng.uniform(-150, -50),
                      rng.uniform(-80, 80), rng.uniform(-30, 30), rng.uniform(-30, 30), 0.0, 0.0])
        out = O.plastic_flow(sc, s, 0.01)
        sig = out[:3].mean()
        J2 = ((out[0] - out[1]) ** 2 + (out[1] - out[2]) ** 2 + (out[2] - out[0]) ** 2) / 6 + \
            out[3] ** 2 + out[4] ** 2 + out[5] ** 2
        Y = math.sqrt(J2) - max(-mu * sig, 0.0)
        assert out[6] >= 0.0
        assert Y <= 1e-9 * abs(sig) + 1e-12
        assert math.isclose(out[7], 0.01 * out[6], rel_tol=1e-14, abs_tol=1e-300)


def test_level_step_is_independent_of_the_patch_layout():
    """The level step of a domain split into uneven patches equals the single-patch step
    bit for bit (exchange fills every ghost cell the stencil reads)."""
    sc = S.slip_weakening(nx=48, ny=24, dx=0.1)
    rng = np.random.default_rng(8)
    U = sc.initial_U()
    U[:, 4:-4, 4:-4] += rng.normal(0, 0.1, U[:, 4:-4, 4:-4].shape)
    B = sc.initial_B()
    U1, B1 = U.copy(), B.copy()
    boxes = [(0, 0, 10, 7), (11, 0, 47, 7), (0, 8, 30, 23), (31, 8, 47, 23)]
    t = 0.0
    for _ in range(5):
        assert O.level_step(sc, U, B, boxes, t, sc.dt()) == 0
        assert O.level_step(sc, U1, B1, [(0, 0, 47, 23)], t, sc.dt()) == 0
        t += sc.dt()
    assert np.array_equal(U[:, 4:-4, 4:-4], U1[:, 4:-4, 4:-4])
    assert np.array_equal(B[:, 4:-4], B1[:, 4:-4])


def test_rupture_propagates_in_the_oracle():
    sc = S.slip_weakening(nx=128, ny=64, dx=0.1)
    U, B = sc.initial_U(), sc.initial_B()
    t = 0.0
    for _ in range(80):
        assert O.level_step(sc, U, B, O.tile_boxes(128, 64, 64), t, sc.dt(), nthreads=4) == 0
        t += sc.dt()
    rt = B[8, 4:-4]
    assert (rt < 1e9).sum() > 30
    assert np.isfinite(U).all()


def test_per_face_friction_in_the_oracle():
    """Per-face a, b, L equal to the scenario's constants reproduce the constant
    run bit for bit; a +-10% field changes the fault's evolution."""
    sc = S.rate_state(nx=48, ny=24, dx=0.1)
    sc.rs.L = 0.002
    rng = np.random.default_rng(12)
    U = sc.initial_U()
    U[:, 4:-4, 4:-4] += rng.normal(0, 0.05, U[:, 4:-4, 4:-4].shape)
    B = sc.initial_B()
    const = np.tile(np.array([sc.rs.a, sc.rs.b, sc.rs.L])[:, None], (1, B.shape[1]))
    hetero = S.friction_field(sc, seed=4001)
    runs = []
    for F in (None, const, hetero):
        Ur, Br = U.copy(), B.copy()
        t = 0.0
        for _ in range(4):
            assert O.level_step(sc, Ur, Br, [(0, 0, 23, 23), (24, 0, 47, 23)], t, sc.dt(), fric=F) == 0
            t += sc.dt()
        runs.append((Ur, Br))
    assert np.array_equal(runs[0][0], runs[1][0]) and np.array_equal(runs[0][1], runs[1][1])
    assert not np.array_equal(runs[0][1][10], runs[2][1][10])


def test_plm_predictor_in_the_oracle():
    """The PLM normal predictor keeps a uniform state uniform and, on a smooth
    perturbation, stays within the second-order agreement of the PPM step;
    fourth-order and second-order slopes differ only slightly."""
    res = {}
    for order, fourth in ((2, 1), (1, 1), (1, 0)):
        sc = S.rate_state(nx=48, ny=24, dx=0.1)
        sc.scheme.normal_pred_order, sc.scheme.use_fourth_order_slopes = order, fourth
        U, B = sc.initial_U(), sc.initial_B()
        U0 = U.copy()
        assert O.level_step(sc, U, B, [(0, 0, 47, 23)], 0.0, sc.dt()) == 0
        far = (slice(None), slice(12, 20), slice(30, 40))      # away from the fault and the nucleation
        assert np.array_equal(U[far], U0[far])
        x = (np.arange(48 + 8) + 0.5) / 48.0
        U = sc.initial_U()
        U[1] += 0.05 * np.sin(2 * np.pi * x)[None, :]
        B = sc.initial_B()
        for k in range(3):
            assert O.level_step(sc, U, B, [(0, 0, 47, 23)], k * sc.dt(), sc.dt()) == 0
        assert np.isfinite(U).all()
        res[(order, fourth)] = U[:, 4:-4, 4:-4]
    ref = np.abs(res[(2, 1)][1]).max()
    assert np.abs(res[(1, 1)][1] - res[(2, 1)][1]).max() < 0.05 * ref
    assert np.abs(res[(1, 1)][1] - res[(1, 0)][1]).max() < 0.05 * ref
    assert not np.array_equal(res[(1, 1)], res[(1, 0)])
