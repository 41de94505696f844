"""Rupture scenarios in the reference decks' units and their initial data.

Each builder returns a `Scenario` holding the C-ABI parameter structs plus the
grid (cells, dx).  Initial data follow the reference's initialisers:
  * U = background stress on both sides, velocities and lambda, gamma zero
    (LEINITF, srcLinElast/LinElastPhysicsF.ChF:1215-1263);
  * rate-and-state B: zeros, rupture time 1e10, psi = psi_init
    (RSIBC::initializeBdry, ibcLinElast/RSIBC.cpp:115-163);
  * slip-weakening B: V, slip_x = 0 and slip_z = 100 as SWIBC::initializeBdry
    sets (ibcLinElast/SWIBC.cpp:121-145); the components it leaves uninitialised
    are set here to 0, with rupture time 1e10.
Units: km, km/s, g/cm^3, GPa, MPa, m/s, m, s.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

from . import _capi as A


@dataclasses.dataclass
class Scenario:
    name: str
    nx: int
    ny: int
    dx: float
    cfl: float
    elastic: A.ElasticParams
    scheme: A.Scheme
    rs: A.RSParams | None = None
    sw: A.SWParams | None = None
    plastic: A.PlasticParams | None = None

    @property
    def nbdry(self) -> int:
        if self.scheme.fault_law == A.TMK_FAULT_RS:
            return A.TMK_RS_NBDRY
        if self.scheme.fault_law == A.TMK_FAULT_SW:
            return A.TMK_SW_NBDRY
        return 0

    def constants(self) -> dict:
        e = self.elastic
        G = e.rho * e.cs * e.cs if e.rho > 0 else e.G
        rho = G / (e.cs * e.cs)
        lam = e.cp * e.cp * rho - 2.0 * G
        return dict(G=G, rho=rho, lam=lam, Zs=rho * e.cs, Zp=rho * e.cp, K=lam + 2.0 * G / 3.0)

    def dt(self) -> float:
        """cfl * dx / max(cs, cp) (MAXWAVESPEEDF, AMRLevelLinElast::advance)."""
        return self.cfl * self.dx / max(self.elastic.cs, self.elastic.cp)

    def background(self) -> np.ndarray:
        e = self.elastic
        side = [0.0, 0.0, 0.0, e.sxx0, e.syy0, e.szz0, e.sxy0, e.sxz0, e.syz0, 0.0, 0.0]
        return np.array(side + side, dtype=np.float64)

    def initial_U(self, lo=(0, 0), hi=None, ghost=A.TMK_NGHOST) -> np.ndarray:
        """State FAB (22, ny+2g, nx+2g) over [lo, hi] grown by `ghost`, set to background."""
        if hi is None:
            hi = (self.nx - 1, self.ny - 1)
        ny = hi[1] - lo[1] + 1 + 2 * ghost
        nx = hi[0] - lo[0] + 1 + 2 * ghost
        U = np.empty((A.TMK_NCOMP, ny, nx), dtype=np.float64)
        U[:] = self.background()[:, None, None]
        return U

    def initial_B(self, xlo=0, xhi=None, ghost=A.TMK_NGHOST) -> np.ndarray | None:
        """Fault FAB (nbdry, nx+2g) over faces [xlo, xhi] grown by `ghost`."""
        if self.scheme.fault_law == A.TMK_FAULT_NONE:
            return None
        if xhi is None:
            xhi = self.nx - 1
        n = xhi - xlo + 1 + 2 * ghost
        if self.scheme.fault_law == A.TMK_FAULT_RS:
            B = np.zeros((A.TMK_RS_NBDRY, n))
            B[9] = 1e10
            B[10] = self.rs.psi_init
        else:
            B = np.zeros((A.TMK_SW_NBDRY, n))
            B[6] = 100.0
            B[8] = 1e10
        return B


def _scheme(fault_law: int, precision: int = A.TMK_PREC_FP64, plasticity: int = 0,
            prim: int = 1, char: int = 0, order: int = 2, bc=(0, 0, 2, 0, 0, 0)) -> A.Scheme:
    s = A.Scheme()
    s.normal_pred_order = order
    s.use_prim_limiting = prim
    s.use_char_limiting = char
    for k in range(6):
        s.boundary_type[k] = bc[k]
    s.fault_law = fault_law
    s.plasticity = plasticity
    s.precision = precision
    s.use_fourth_order_slopes = 1     # the decks' setting (used by the PLM predictor only)
    return s


def _elastic(cs=3.464, cp=6.0, rho=2.670, sxx0=0.0, syy0=-120.0, szz0=0.0, sxy0=70.0, sxz0=0.0,
             syz0=0.0) -> A.ElasticParams:
    e = A.ElasticParams()
    e.cs, e.cp, e.G, e.rho = cs, cp, 0.0, rho
    e.sxx0, e.syy0, e.szz0, e.sxy0, e.sxz0, e.syz0 = sxx0, syy0, szz0, sxy0, sxz0, syz0
    return e


def plastic_background(syy0: float, sxy0: float, psi_deg: float) -> tuple[float, float]:
    """sxx0 and szz0 of a deck with physics.plas_Psi (the angle of the largest
    compressive stress to the fault): the rule of execLinElast/amrGodunov.cpp:482-495."""
    if psi_deg == 45:
        sxx0 = syy0
    else:
        sxx0 = (1.0 - 2.0 * sxy0 / (syy0 * math.tan(2.0 * (math.pi * psi_deg / 180.0)))) * syy0
    return sxx0, (sxx0 + syy0) / 2.0


def psi_steady(tau: float, sn: float, V: float, a: float, V0: float, Zs: float) -> float:
    """State psi at which slip rate V is steady under shear tau and normal stress sn:
    tau - Zs/2 V = sn a asinh(V/(2 V0) exp(psi/a))."""
    return a * math.log((2.0 * V0 / V) * math.sinh((tau - 0.5 * Zs * V) / (a * sn)))


def slip_weakening(nx=512, ny=256, dx=0.1, precision=A.TMK_PREC_FP64,
                   layout=A.TMK_SW_LAYOUT_OFFSET11, cfl=0.9, plasticity=False,
                   nuc_tau=11.6, nuc_half_width=1.5, cohesion=0.0, plas_psi=None) -> Scenario:
    """Slip-weakening planar fault at y=0 (the 512x256, dx=0.1 km CPU-runnable workload):
    mu_s=0.677, mu_d=0.525, Dc=0.4 m, sn=120 MPa, tau=70 MPa, a 3 km nucleation
    window at 81.6 MPa (11.6 MPa excess), friction box covering the whole fault."""
    sw = A.SWParams()
    sw.fs, sw.fd, sw.dw, sw.smooth = 0.677, 0.525, 0.4, 0.0
    sw.num_patches = 1
    sw.xc[0], sw.xw[0], sw.zc[0], sw.zw[0], sw.tau[0] = 0.0, nuc_half_width, 0.0, nuc_half_width, nuc_tau
    sw.fric_box_center[0], sw.fric_box_center[1] = nx * dx / 2.0, 0.0
    sw.fric_box_width[0], sw.fric_box_width[1] = 1e3, 1e3
    sw.outside_friction = 1e4
    sw.rupture_threshold = 0.001
    sw.layout = layout
    pl = None
    if plasticity:
        pl = plastic_params(cohesion=cohesion)
    e = _elastic()
    if plas_psi is not None:       # the deck's plas_Psi sets the background's normal stresses
        e.sxx0, e.szz0 = plastic_background(e.syy0, e.sxy0, plas_psi)
    return Scenario("slip_weakening", nx, ny, dx, cfl, e,
                    _scheme(A.TMK_FAULT_SW, precision, int(plasticity)), sw=sw, plastic=pl)


def rate_state(nx=2048, ny=1024, dx=0.1, precision=A.TMK_PREC_FP64,
               state_law=A.TMK_RS_AGING_LAW, cfl=0.9, plasticity=False, V_init=1e-12) -> Scenario:
    """Rate-and-state planar fault at y=0 (the 2048x1024, dx=0.1 km benchmark workload):
    a=0.008, b=0.012, L=0.02 m, f0=0.6, V0=1e-6 m/s, initial V=1e-12 m/s, Gaussian
    shear nucleation of 25 MPa amplitude and 3 km width at the fault centre."""
    e = _elastic()
    sc = Scenario("rate_state", nx, ny, dx, cfl, e, _scheme(A.TMK_FAULT_RS, precision, int(plasticity)))
    c = sc.constants()
    rs = A.RSParams()
    rs.r0, rs.x0, rs.y0, rs.nsig, rs.ntime = 3.0, nx * dx / 2.0, 0.0, 25.0, 0.0
    rs.a, rs.b, rs.V0, rs.f0, rs.L = 0.008, 0.012, 1e-6, 0.6, 0.02
    rs.fw, rs.Vw, rs.fexp = 0.1, 0.1, -1.0
    rs.ramp_x, rs.ramp_w, rs.ramp_a, rs.ramp_Vw = 0.0, 1e40, 0.0, 0.0
    rs.rupture_threshold = 0.001
    rs.psi_init = psi_steady(e.sxy0, -e.syy0, V_init, rs.a, rs.V0, c["Zs"])
    rs.state_law = state_law
    sc.rs = rs
    if plasticity:
        sc.plastic = plastic_params()
    return sc


def plastic_params(mu=math.sin(0.75), eta_time=0.03, G=None, cohesion=0.0) -> A.PlasticParams:
    """Drucker-Prager: plas_mu, plas_beta = plas_mu/2 (execLinElast/amrGodunov.cpp:514),
    plas_eta = eta_time * G (viscoplastic relaxation time eta/G).  A cohesion c
    (MPa) enters as the yield term b = c cos(phi) with mu = sin(phi); the
    reference hard-wires b = 0 (srcLinElast/PlasticPhysicsF.ChF:19), so c > 0 is
    an extension."""
    if G is None:
        G = 2.670 * 3.464 ** 2
    p = A.PlasticParams()
    p.mu, p.beta, p.eta, p.h = mu, mu / 2.0, eta_time * G, 0.0
    p.b = cohesion * math.cos(math.asin(mu))
    return p


# ------------------------------------------------------------------ ensembles
ENSEMBLE_GRIDS = ((256, 128), (512, 256), (1024, 512))


def lognormal_field(n: int, dx: float, corr_len: float, mean: float, s: float, seed: int) -> np.ndarray:
    """mean * exp(g - s^2/2) on n cells of width dx, with g a stationary Gaussian
    field of variance s^2 and exponential covariance s^2 exp(-|r|/corr_len).
    Spectral synthesis by circulant embedding (Dietrich & Newsam 1997) on a
    periodic grid of 2n cells, whose eigenvalues are non-negative for this
    covariance in one dimension."""
    m = 2 * n
    j = np.arange(m)
    r = np.minimum(j, m - j) * dx
    lam = np.fft.fft(s * s * np.exp(-r / corr_len)).real
    lam = np.maximum(lam, 0.0)
    rng = np.random.default_rng(seed)
    z = rng.standard_normal(m) + 1j * rng.standard_normal(m)
    g = np.fft.fft(np.sqrt(lam / m) * z).real[:n]
    return mean * np.exp(g - 0.5 * s * s)


def ensemble_member(k: int, precision=A.TMK_PREC_MIXED, dx=0.1, grids=ENSEMBLE_GRIDS, V_init=1e-12):
    """Scenario k of the seeded rate-and-state ensemble: grid drawn from `grids`,
    a ~ U[0.006, 0.012], b - a ~ U[0.002, 0.006], L ~ U[0.01, 0.05] m (seed
    5000 + k), and a shear prestress tau0(x) = 70 exp(g(x) - s^2/2) MPa along
    strike, g Gaussian with exponential covariance, correlation length 1 km and
    s = 0.1 (seed 6000 + k).  Returns (scenario, tau0 per fault face)."""
    rng = np.random.default_rng(5000 + k)
    nx, ny = grids[int(rng.integers(len(grids)))]
    a = float(rng.uniform(0.006, 0.012))
    ba = float(rng.uniform(0.002, 0.006))
    L = float(rng.uniform(0.01, 0.05))
    sc = rate_state(nx=nx, ny=ny, dx=dx, precision=precision, V_init=V_init)
    sc.rs.a, sc.rs.b, sc.rs.L = a, a + ba, L
    sc.rs.psi_init = psi_steady(sc.elastic.sxy0, -sc.elastic.syy0, V_init, a, sc.rs.V0, sc.constants()["Zs"])
    tau0 = lognormal_field(nx, dx, 1.0, 70.0, 0.1, 6000 + k)
    return sc, tau0


def prestressed_state(sc: Scenario, tau0: np.ndarray, V_init=1e-12):
    """Domain-wide U and B of a rate-and-state scenario whose shear stress is
    tau0(x) in every row (both sides) and whose state psi is steady at V_init
    under it, face by face."""
    g = A.TMK_NGHOST
    U = sc.initial_U()
    B = sc.initial_B()
    t = np.pad(np.asarray(tau0, dtype=np.float64), g, mode="edge")
    for side in (0, 11):
        U[side + 6] = t[None, :]
    sn = -sc.elastic.syy0
    Zs = sc.constants()["Zs"]
    B[10] = [psi_steady(float(ti), sn, V_init, sc.rs.a, sc.rs.V0, Zs) for ti in t]
    return U, B


def friction_field(sc: Scenario, seed: int = 4001, amp: float = 0.1, refine: int = 1) -> np.ndarray:
    """Per-face rate-and-state (a, b, L) = nominal x (1 + U(-amp, amp)), drawn on
    the scenario's nx faces (seed `seed`), each face's three values independent.
    `refine` > 1 gives the same field on a level refined by that ratio (every
    fine face takes its coarse face's values).  Returned over the faces grown
    by TMK_NGHOST (edge values repeated), shape (3, nx*refine + 8): the layout
    of LinElastLevelGodunov.set_level_friction."""
    rng = np.random.default_rng(seed)
    nom = np.array([sc.rs.a, sc.rs.b, sc.rs.L])[:, None]
    F = nom * (1.0 + rng.uniform(-amp, amp, size=(3, sc.nx)))
    if refine > 1:
        F = np.repeat(F, refine, axis=1)
    return np.pad(F, ((0, 0), (A.TMK_NGHOST, A.TMK_NGHOST)), mode="edge")
