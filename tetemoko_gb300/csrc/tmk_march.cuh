// tmk_march.cuh -- column-marching volume kernel.
//
// A warp owns 32 adjacent columns of a patch (28 updated columns plus a
// 2-column halo on each side) and streams up a run of rows.  Per row it
// computes the x predictor (each lane's neighbours read from the row's copy in
// shared memory, which also holds the column one beyond the warp on either
// side: the outermost slopes need them, and with them a 2-column halo is
// enough for the 3-cell stencil of one update) and the y predictor
// (a rolling window of rows in registers), the first-pass Riemann states,
// the transverse corrections, the final Riemann states, the fluxes and the
// conservative update -- the CTU sequence of LinElastPatchGodunov::computeWHalf
// and LinElastPhysics::computeUpdate (srcLinElast/LinElastPatchGodunov.cpp:174-469)
// -- emitting one updated row per step, three rows behind the loads.
//
// The state of the two fault sides is packed into one pair per component
// (.x = side 1, .y = side 2; the y direction of side 2 is mirrored, rv = -1),
// so the linear algebra runs as packed FP32x2 instructions in the FP32 form.
// The components split into two groups that never mix inside the volume:
//   in-plane  (vx vy sxx syy szz sxy): a P-wave pair, an S-wave pair and the
//             two normal stresses tied to the P-wave stress by lam/(lam+2G);
//   antiplane (vz sxz syz): an S-wave pair and one stress with zero speed.
// The characteristic transforms, the PPM tracing (Colella & Woodward 1984
// eq. 1.12, written as a*w_near + b*w_far with a = (1-s)^2, b = s^2 - s) and
// the syntheses of srcLinElast/LinElastPhysicsF.ChF:359-555 are applied per
// wave pair.
#pragma once
#include "tmk_device.cuh"
#include "tmk_kernels.cuh"

namespace tmk {

// ------------------------------------------------------------ pair arithmetic
template <typename T> struct PairOf;
template <> struct PairOf<float> { using P = float2; };
template <> struct PairOf<double> { using P = double2; };

TMK_HD float2 mk2(float a, float b) { return make_float2(a, b); }
TMK_HD double2 mk2(double a, double b) { return make_double2(a, b); }
TMK_D float2 padd(float2 a, float2 b) { return __fadd2_rn(a, b); }
TMK_D float2 pmul(float2 a, float2 b) { return __fmul2_rn(a, b); }
TMK_D float2 pfma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
TMK_D float2 psub(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }
TMK_D double2 padd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
TMK_D double2 pmul(double2 a, double2 b) { return make_double2(a.x * b.x, a.y * b.y); }
TMK_D double2 pfma(double2 a, double2 b, double2 c) { return make_double2(a.x * b.x + c.x, a.y * b.y + c.y); }
TMK_D double2 psub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
template <typename P> TMK_D P pneg(P a) { return pmul(a, mk2(decltype(a.x)(-1), decltype(a.x)(-1))); }

TMK_D float2 shfl_up2(float2 v, int d) {
  return make_float2(__shfl_up_sync(0xffffffffu, v.x, d), __shfl_up_sync(0xffffffffu, v.y, d));
}
TMK_D float2 shfl_dn2(float2 v, int d) {
  return make_float2(__shfl_down_sync(0xffffffffu, v.x, d), __shfl_down_sync(0xffffffffu, v.y, d));
}
TMK_D double2 shfl_up2(double2 v, int d) {
  return make_double2(__shfl_up_sync(0xffffffffu, v.x, d), __shfl_up_sync(0xffffffffu, v.y, d));
}
TMK_D double2 shfl_dn2(double2 v, int d) {
  return make_double2(__shfl_down_sync(0xffffffffu, v.x, d), __shfl_down_sync(0xffffffffu, v.y, d));
}

// ------------------------------------------------------------ groups and roles
template <int G> struct Grp;
template <> struct Grp<0> {   // in-plane
  static constexpr int N = 6;
  TMK_HD static constexpr int glob(int k) { return k == 0 ? 0 : k == 1 ? 1 : k == 2 ? 3 : k == 3 ? 4 : k == 4 ? 5 : 6; }
};
template <> struct Grp<1> {   // antiplane
  static constexpr int N = 3;
  TMK_HD static constexpr int glob(int k) { return k == 0 ? 2 : k == 1 ? 7 : 8; }
};

// Wave roles of the group's components in direction D (indices into the group):
//   P pair (vP, sP), S pair (vS, sS), zero-speed components coupled to sP
//   (zc0, zc1: normal stresses, z - lam/(lam+2G) sP is invariant), and a
//   zero-speed component with no coupling (zf).
template <int G, int D> struct Role;
template <> struct Role<0, 0> { static constexpr bool hasP = true, hasZc = true, hasZf = false;
  static constexpr int vP = 0, sP = 2, vS = 1, sS = 5, zc0 = 3, zc1 = 4, zf = 0; };
template <> struct Role<0, 1> { static constexpr bool hasP = true, hasZc = true, hasZf = false;
  static constexpr int vP = 1, sP = 3, vS = 0, sS = 5, zc0 = 4, zc1 = 2, zf = 0; };
template <> struct Role<1, 0> { static constexpr bool hasP = false, hasZc = false, hasZf = true;
  static constexpr int vP = 0, sP = 0, vS = 0, sS = 1, zc0 = 0, zc1 = 0, zf = 2; };
template <> struct Role<1, 1> { static constexpr bool hasP = false, hasZc = false, hasZf = true;
  static constexpr int vP = 0, sP = 0, vS = 0, sS = 2, zc0 = 0, zc1 = 0, zf = 1; };

// Components of a group whose direction-D states feed no flux and no
// transverse term: the zero-speed components of the direction (the normal
// stresses tied to the P-wave stress, the uncoupled stress).  RIEMANNF, the
// edge conditions, GETFLUXF and GETADWDXF read only the P and S wave pairs of
// a face state, and those are formed from the wave pairs of the cell states
// alone, so these components of the predicted states, of the face states and
// of a transverse correction aimed at direction D are never read: the kernels
// skip them (szz, for instance, is updated from the fluxes of the velocities
// but feeds no face state in either direction).
template <int G, int D> TMK_HD constexpr bool live(int c) {
  using R = Role<G, D>;
  return !((R::hasZc && (c == R::zc0 || c == R::zc1)) || (R::hasZf && c == R::zf));
}

// Packed constants of one direction.  A packed FP32x2 instruction takes a
// constant operand straight from the parameter bank only when both halves are
// the same scalar (a broadcast); a pair of two values has to be loaded into
// registers at each use once the registers are full.  So every constant is
// also kept as its side-1 scalar (the s* fields): in x, and for the constants
// that do not change sign with the mirrored y direction of side 2, the
// kernels build the pair from that scalar (kc, ke); only the y-direction
// constants with rv (side 2 = -side 1) are used as pairs.
template <typename T>
struct MK {
  using P = typename PairOf<T>::P;
  P ZpE, ZsE;          // characteristic w = s +- ZE v (ZE = rv Z)
  P nZpE, nZsE;        // -ZE
  P hZpE, hZsE;        // synthesis v = (w- - w+) * rv/(2Z)
  P half, r, nr;       // 1/2, lam/(lam+2G), -lam/(lam+2G)
  P aP, bP, aS, bS;    // PPM tracing coefficients of the P and S speeds
  P f_irho, f_l2g, f_lam, f_G;   // GETFLUXF: -rv * {1/rho, lam+2G, lam, G}
  P a_irho, a_l2g, a_lam, a_G;   // GETADWDXF: -rv*scale * {...}
  // side-1 scalars of the pairs above
  T sZpE, sZsE, snZpE, snZsE, shZpE, shZsE, saP, sbP, saS, sbS;
  T sf_irho, sf_l2g, sf_lam, sf_G, sa_irho, sa_l2g, sa_lam, sa_G;
  TMK_HD void load(const DevParams& p, int D, double dtdx, double scale) {
    const T s2 = (D == 1) ? T(-1) : T(1);       // rv of side 2
    ZpE = mk2((T)p.Zp, (T)(s2 * p.Zp)); ZsE = mk2((T)p.Zs, (T)(s2 * p.Zs));
    nZpE = mk2((T)-p.Zp, (T)(-s2 * p.Zp)); nZsE = mk2((T)-p.Zs, (T)(-s2 * p.Zs));
    hZpE = mk2((T)(0.5 / p.Zp), (T)(s2 * 0.5 / p.Zp)); hZsE = mk2((T)(0.5 / p.Zs), (T)(s2 * 0.5 / p.Zs));
    half = mk2(T(0.5), T(0.5));
    const T rr = (T)(p.lam / (p.lam + 2.0 * p.G));
    r = mk2(rr, rr);
    nr = mk2(-rr, -rr);
    const double sp = p.cp * dtdx, ss = p.cs * dtdx;
    const T ap = (T)((1.0 - sp) * (1.0 - sp)), bp = (T)(sp * sp - sp);
    const T as = (T)((1.0 - ss) * (1.0 - ss)), bs = (T)(ss * ss - ss);
    aP = mk2(ap, ap); bP = mk2(bp, bp); aS = mk2(as, as); bS = mk2(bs, bs);
    const double m1 = -1.0, m2 = -s2;
    f_irho = mk2((T)(m1 / p.rho), (T)(m2 / p.rho));
    f_l2g = mk2((T)(m1 * (p.lam + 2.0 * p.G)), (T)(m2 * (p.lam + 2.0 * p.G)));
    f_lam = mk2((T)(m1 * p.lam), (T)(m2 * p.lam));
    f_G = mk2((T)(m1 * p.G), (T)(m2 * p.G));
    a_irho = mk2((T)(m1 * scale / p.rho), (T)(m2 * scale / p.rho));
    a_l2g = mk2((T)(m1 * scale * (p.lam + 2.0 * p.G)), (T)(m2 * scale * (p.lam + 2.0 * p.G)));
    a_lam = mk2((T)(m1 * scale * p.lam), (T)(m2 * scale * p.lam));
    a_G = mk2((T)(m1 * scale * p.G), (T)(m2 * scale * p.G));
    sZpE = ZpE.x; sZsE = ZsE.x; snZpE = nZpE.x; snZsE = nZsE.x; shZpE = hZpE.x; shZsE = hZsE.x;
    saP = ap; sbP = bp; saS = as; sbS = bs;
    sf_irho = f_irho.x; sf_l2g = f_l2g.x; sf_lam = f_lam.x; sf_G = f_G.x;
    sa_irho = a_irho.x; sa_l2g = a_l2g.x; sa_lam = a_lam.x; sa_G = a_G.x;
  }
};

// Constant `name` of direction D as a pair: in x a broadcast of its scalar,
// in y the stored pair (side 2 = -side 1 for the constants carrying rv).
template <int D, typename T>
TMK_D typename PairOf<T>::P kc_(const typename PairOf<T>::P& pair, T s) {
  if constexpr (D == 0) return mk2(s, s);
  else return pair;
}
#define KC(name) kc_<D, T>(k.name, k.s##name)
// a constant with the same value on both sides in either direction
#define KE(name) mk2(k.s##name, k.s##name)
#define KHALF mk2(T(0.5), T(0.5))

// Everything the marching kernel needs that is uniform over a launch (all
// patches of a level share the scenario, dt and dx).  Built on the host and
// passed by value as a __grid_constant__ parameter, so the kernel reads the
// constants from the parameter bank instead of holding ~90 of them in
// registers through the row loop.
template <typename T>
struct MarchConst {
  using P = typename PairOf<T>::P;
  MK<T> kx, ky;
  P bg[9];           // background of the evolving components (.x side 1, .y side 2)
  P sc;              // -dt/dx
  int plim, clim, lim, ppm;
  int xout_lo, xout_hi, yout_lo, yout_hi;
  void* stash[2];    // row-0 intermediates of the fault-row items, per component group
  const int4* caps[2];   // coarse-fine faces each group's items store (row, kind, lane, slot)
  // Drucker-Prager return of a plastic level when it is fused into the
  // in-plane group's stores (the antiplane group's updated stresses are stored
  // first); the level's tuning sets `plastic`
  PlasticK<T> pk;
  T pdt;
  int plastic;
  TMK_HD void load(const DevParams& p, double dt, double dx) {
    const double dtdx = dt / dx;
    kx.load(p, 0, dtdx, -(1.0 / 2.0) * dt / dx);
    ky.load(p, 1, dtdx, -(1.0 / 2.0) * dt / dx);
    for (int c = 0; c < 9; ++c) bg[c] = mk2((T)p.bg[c], (T)p.bg[11 + c]);
    sc = mk2((T)(-dt / dx), (T)(-dt / dx));
    plim = p.prim_lim != 0; clim = p.char_lim != 0; lim = plim || clim; ppm = p.order != 0;
    xout_lo = p.bc[0] == 0; xout_hi = p.bc[1] == 0; yout_lo = p.bc[2] == 0; yout_hi = p.bc[3] == 0;
    plastic = 0;
    pk.load(p);
    pdt = (T)dt;
  }
};

// ---- limiters on pairs (differences packed, the nonlinear part per half)
TMK_D float copysg(float a, float b) { return copysignf(a, b); }
TMK_D double copysg(double a, double b) { return copysign(a, b); }

// van Leer: sign(dc) min(|dc|, 2|dl|, 2|dr|) when dl dr > 0, else 0 (dl2, dr2:
// the doubled differences, exact; one three-input minimum)
template <typename T> TMK_D T vl1(T dl2, T dr2, T dc, T prod) {
  const T t = fmin(fmin(fabs(dc), fabs(dl2)), fabs(dr2));
  return prod > T(0) ? copysg(t, dc) : T(0);
}

// Limited slope of the middle value.  A missing neighbour (outside the
// domain) stands for the reflection 2 w0 - w_other, which makes the two
// one-sided differences equal: the centred formula becomes the one-sided
// difference the reference uses there.
template <typename P> TMK_D P slope2(P wm, P w0, P wp, bool hasL, bool hasR, bool limit) {
  using T = decltype(wm.x);
  const P half = mk2(T(0.5), T(0.5));
  P dl = psub(w0, wm), dr = psub(wp, w0);
  if (!hasL) dl = dr;
  if (!hasR) dr = dl;
  const P dc = pmul(half, padd(dl, dr));
  if (!limit) return dc;
  const P prod = pmul(dl, dr);
  const P dl2 = padd(dl, dl), dr2 = padd(dr, dr);
  return mk2(vl1(dl2.x, dr2.x, dc.x, prod.x), vl1(dl2.y, dr2.y, dc.y, prod.y));
}

// PPM limiter (Colella & Woodward 1984 eq. 1.10): both deltas zero at an
// extremum, otherwise each clipped to twice the other's magnitude.
template <typename T> TMK_D T clampabs(T v, T b) { return fmin(fmax(v, -fabs(b)), fabs(b)); }
template <typename P> TMK_D void limit2(P& m, P& p) {
  using T = decltype(m.x);
  const P two = mk2(T(2), T(2));
  const P m2 = pmul(two, m), p2 = pmul(two, p), prod = pmul(m, p);
  const T amx = clampabs(m.x, p2.x), apx = clampabs(p.x, m2.x);
  const T amy = clampabs(m.y, p2.y), apy = clampabs(p.y, m2.y);
  m.x = prod.x < T(0) ? amx : T(0); p.x = prod.x < T(0) ? apx : T(0);
  m.y = prod.y < T(0) ? amy : T(0); p.y = prod.y < T(0) ? apy : T(0);
}

// interior PPM face value between cells a (lower) and b: (a+b)/2 - (sb - sa)/6
template <typename T, typename P> TMK_D P face2(P a, P b, P sa, P sb) {
  const P h = mk2(T(0.5), T(0.5)), m6 = mk2(T(-1.0 / 6.0), T(-1.0 / 6.0));
  return pfma(psub(sb, sa), m6, pmul(h, padd(a, b)));
}

// PPM normal predictor of a group in direction D from the unlimited face
// deltas dm (lo face) and dp (hi face) of each component; WM, WP = w + traced.
template <int G, int D, typename T>
TMK_D void predict(const MK<T>& k, const typename PairOf<T>::P* w, typename PairOf<T>::P* dm,
                   typename PairOf<T>::P* dp, bool plim, bool clim, typename PairOf<T>::P* WM,
                   typename PairOf<T>::P* WP) {
  using P = typename PairOf<T>::P;
  using R = Role<G, D>;
  constexpr int N = Grp<G>::N;
  if (plim) {
#pragma unroll
    for (int c = 0; c < N; ++c)
      if (live<G, D>(c)) limit2(dm[c], dp[c]);
  }
  // S wave pair
  {
    P nm = pfma(KC(ZsE), dm[R::vS], dm[R::sS]), pm = pfma(KC(nZsE), dm[R::vS], dm[R::sS]);
    P np = pfma(KC(ZsE), dp[R::vS], dp[R::sS]), pp = pfma(KC(nZsE), dp[R::vS], dp[R::sS]);
    if (clim) { limit2(nm, np); limit2(pm, pp); }
    P nmt = pfma(KE(aS), nm, pmul(KE(bS), np));       // w- traced to the lo face
    P ppt = pfma(KE(aS), pp, pmul(KE(bS), pm));       // w+ traced to the hi face
    WM[R::sS] = padd(w[R::sS], pmul(KHALF, padd(nmt, pm)));
    WM[R::vS] = padd(w[R::vS], pmul(KC(hZsE), psub(nmt, pm)));
    WP[R::sS] = padd(w[R::sS], pmul(KHALF, padd(np, ppt)));
    WP[R::vS] = padd(w[R::vS], pmul(KC(hZsE), psub(np, ppt)));
  }
  if constexpr (R::hasP) {
    P nm = pfma(KC(ZpE), dm[R::vP], dm[R::sP]), pm = pfma(KC(nZpE), dm[R::vP], dm[R::sP]);
    P np = pfma(KC(ZpE), dp[R::vP], dp[R::sP]), pp = pfma(KC(nZpE), dp[R::vP], dp[R::sP]);
    if (clim) { limit2(nm, np); limit2(pm, pp); }
    P nmt = pfma(KE(aP), nm, pmul(KE(bP), np));
    P ppt = pfma(KE(aP), pp, pmul(KE(bP), pm));
    P sPm = pmul(KHALF, padd(nmt, pm)), sPp = pmul(KHALF, padd(np, ppt));
    WM[R::sP] = padd(w[R::sP], sPm);
    WM[R::vP] = padd(w[R::vP], pmul(KC(hZpE), psub(nmt, pm)));
    WP[R::sP] = padd(w[R::sP], sPp);
    WP[R::vP] = padd(w[R::vP], pmul(KC(hZpE), psub(np, ppt)));
  }
  // the zero-speed components of direction D are not read (live<G, D>)
#pragma unroll
  for (int c = 0; c < Grp<G>::N; ++c)
    if (!live<G, D>(c)) { WM[c] = mk2(T(0), T(0)); WP[c] = mk2(T(0), T(0)); }
}

// RIEMANNF for a group: L = state left of the face, Rt = right
template <int G, int D, typename T>
TMK_D void riem(const MK<T>& k, const typename PairOf<T>::P* L, const typename PairOf<T>::P* Rt,
                typename PairOf<T>::P* g) {
  using P = typename PairOf<T>::P;
  using R = Role<G, D>;
  {
    P wpos = pfma(KC(nZsE), L[R::vS], L[R::sS]);
    P wneg = pfma(KC(ZsE), Rt[R::vS], Rt[R::sS]);
    g[R::sS] = pmul(KHALF, padd(wneg, wpos));
    g[R::vS] = pmul(KC(hZsE), psub(wneg, wpos));
  }
  if constexpr (R::hasP) {
    P wpos = pfma(KC(nZpE), L[R::vP], L[R::sP]);
    P wneg = pfma(KC(ZpE), Rt[R::vP], Rt[R::sP]);
    P s = pmul(KHALF, padd(wneg, wpos));
    g[R::sP] = s;
    g[R::vP] = pmul(KC(hZpE), psub(wneg, wpos));
  }
  // zero-speed components of the face state: not read (live<G, D>)
#pragma unroll
  for (int c = 0; c < Grp<G>::N; ++c)
    if (!live<G, D>(c)) g[c] = mk2(decltype(L[0].x)(0), decltype(L[0].x)(0));
}

// Background state of a group, read from the launch constants by group index.
template <int G, typename P>
struct BgView {
  const P* all;   // the 9 evolving components
  TMK_D P operator[](int c) const { return all[Grp<G>::glob(c)]; }
};

// LINELASTOUTBCF / LINELASTFREEBCF for a group.  lo: the inside state is the
// cell above/right of the face; SHF keeps the reference's velocity-minus-stress form.
template <int G, int D, typename T>
TMK_D void edge2(const MK<T>& k, bool lo, bool outflow, const typename PairOf<T>::P* Wi,
                 const BgView<G, typename PairOf<T>::P>& bg, typename PairOf<T>::P* g) {
  using P = typename PairOf<T>::P;
  using R = Role<G, D>;
  {
    P wneg, wpos;
    if (lo) {
      wneg = pfma(KC(ZsE), Wi[R::vS], Wi[R::sS]);
      wpos = outflow ? pfma(KC(nZsE), bg[R::vS], bg[R::sS]) : pneg(wneg);
    } else {
      wpos = pfma(KC(nZsE), Wi[R::vS], Wi[R::sS]);
      wneg = outflow ? pfma(KC(ZsE), bg[R::vS], bg[R::sS]) : pneg(wpos);
    }
    g[R::sS] = pmul(KHALF, padd(wneg, wpos));
    g[R::vS] = pmul(KC(hZsE), psub(wneg, wpos));
  }
  if constexpr (R::hasP) {
    P wneg, wpos;
    if (lo) {
      wneg = pfma(KC(ZpE), Wi[R::vP], Wi[R::sP]);
      wpos = outflow ? pfma(KC(nZpE), bg[R::vP], bg[R::sP]) : pneg(wneg);
    } else {
      wpos = pfma(KC(nZpE), Wi[R::vP], Wi[R::sP]);
      wneg = outflow ? pfma(KC(ZpE), bg[R::vP], bg[R::sP]) : pneg(wpos);
    }
    P s = pmul(KHALF, padd(wneg, wpos));
    g[R::sP] = s;
    g[R::vP] = pmul(KC(hZpE), psub(wneg, wpos));
  }
  // zero-speed components (the reference's SHF terms): not read (live<G, D>)
#pragma unroll
  for (int c = 0; c < Grp<G>::N; ++c)
    if (!live<G, D>(c)) g[c] = mk2(T(0), T(0));
}

// GETFLUXF for a group
template <int G, int D, typename T>
TMK_D void flux2(const MK<T>& k, const typename PairOf<T>::P* g, typename PairOf<T>::P* F) {
  using R = Role<G, D>;
  F[R::vS] = pmul(KC(f_irho), g[R::sS]);
  F[R::sS] = pmul(KC(f_G), g[R::vS]);
  if constexpr (R::hasP) {
    F[R::vP] = pmul(KC(f_irho), g[R::sP]);
    F[R::sP] = pmul(KC(f_l2g), g[R::vP]);
    F[R::zc0] = pmul(KC(f_lam), g[R::vP]);
    F[R::zc1] = pmul(KC(f_lam), g[R::vP]);
  }
  if constexpr (R::hasZf) F[R::zf] = mk2(decltype(g[0].x)(0), decltype(g[0].x)(0));
}

// GETADWDXF increment from the face states at the hi (h) and lo (l) faces, added to q1 and q2
template <int G, int D, typename T>
TMK_D void adw2(const MK<T>& k, const typename PairOf<T>::P* h, const typename PairOf<T>::P* l,
                typename PairOf<T>::P* q1, typename PairOf<T>::P* q2) {
  using P = typename PairOf<T>::P;
  using R = Role<G, D>;
  {
    P a = pmul(KC(a_irho), psub(h[R::sS], l[R::sS]));
    q1[R::vS] = padd(q1[R::vS], a); q2[R::vS] = padd(q2[R::vS], a);
    P b = pmul(KC(a_G), psub(h[R::vS], l[R::vS]));
    q1[R::sS] = padd(q1[R::sS], b); q2[R::sS] = padd(q2[R::sS], b);
  }
  if constexpr (R::hasP) {
    P a = pmul(KC(a_irho), psub(h[R::sP], l[R::sP]));
    q1[R::vP] = padd(q1[R::vP], a); q2[R::vP] = padd(q2[R::vP], a);
    P dv = psub(h[R::vP], l[R::vP]);
    P b = pmul(KC(a_l2g), dv);
    q1[R::sP] = padd(q1[R::sP], b); q2[R::sP] = padd(q2[R::sP], b);
    // the targets are states of the other direction: their components that
    // are zero-speed there are not read
    P c = pmul(KC(a_lam), dv);
    if constexpr (live<G, 1 - D>(R::zc0)) { q1[R::zc0] = padd(q1[R::zc0], c); q2[R::zc0] = padd(q2[R::zc0], c); }
    if constexpr (live<G, 1 - D>(R::zc1)) { q1[R::zc1] = padd(q1[R::zc1], c); q2[R::zc1] = padd(q2[R::zc1], c); }
  }
}

// ---------------------------------------------------------------- the kernel
// A strip of MARCH_COLS columns of a patch by the rows [y0, y1].  fslot >= 0
// marks the first item of a strip on the fault row: its row 0 needs the fault
// kernel's results, so the kernel leaves that row to march_fault_row_kernel
// and keeps what it needs in stash slot fslot.
// [cap0, cap0+ncap) are the item's entries in its group's capture list.
struct MarchItem { int patch, x0, y0, y1, fslot, cap0, ncap; };
// vectors a fault-row item keeps for its row 0 (x states, first-pass y face 1,
// final y flux 1, old state)
constexpr int MARCH_STASH_VECS = 5;

constexpr int MARCH_COLS = 28;   // updated columns per warp
constexpr int MARCH_HALO = 2;    // halo lanes on either side (lane l holds column x0 - 2 + l)
constexpr int MARCH_WARPS = 4;   // warps per CTA

// Per-row vectors a lane carries from row to row in shared memory rather than
// registers: the x states of row q-1 (WMx, WPx), the first-pass y face q-1
// (H1y), the final y flux q-1 (Fy), the old state of row q-1 (Wold), the
// y-predicted and corrected states of row q-1 (WPy, WPcy), and the y slope
// and lo-face value of row q (Sy, Fyf).  Each keeps only the components that
// are read: the x states the components live in x, the y states and faces
// those live in y.  The FP64 form keeps the last four in registers: in shared
// memory its in-plane CTA would need 131 KB, one CTA per SM.
enum MarchCarry { kWMx = 0, kWPx, kH1y, kFy, kWold, kWPy, kWPcy, kSy, kFyf, kNumCarry };
template <int G>
TMK_HD constexpr bool carry_needed(int v, int c) {
  return (v == kWMx || v == kWPx) ? live<G, 0>(c) : (v == kFy || v == kWold) ? true : live<G, 1>(c);
}
template <typename T>
TMK_HD constexpr bool carry_in_smem(int v) { return v < kWPy || sizeof(T) == 4; }
// position of (vector v, component c) among the shared-memory slots of a lane
template <typename T, int G>
TMK_HD constexpr int carry_slot(int v, int c) {
  int k = 0;
  for (int vv = 0; vv < v; ++vv)
    for (int cc = 0; cc < Grp<G>::N; ++cc) k += (carry_in_smem<T>(vv) && carry_needed<G>(vv, cc)) ? 1 : 0;
  for (int cc = 0; cc < c; ++cc) k += carry_needed<G>(v, cc) ? 1 : 0;
  return k;
}
template <typename T, int G>
TMK_HD constexpr int carry_slots() { return carry_slot<T, G>(kNumCarry, 0); }
// Rows q..q+2 of the rolling window plus the row in flight live in a per-warp
// ring of shared memory filled by cp.async; slot = row & 3.  A ring row holds
// MARCH_RW entries per component: the column left of lane 0, the warp's 32
// columns, the column right of lane 31.
constexpr int MARCH_RING = 4;
constexpr int MARCH_RW = 34;
template <typename T, int G>
constexpr size_t march_warp_pairs() {
  return (size_t)carry_slots<T, G>() * 32 + (size_t)MARCH_RING * Grp<G>::N * MARCH_RW;
}
template <typename T, int G>
constexpr size_t march_smem_bytes() {
  return (size_t)MARCH_WARPS * march_warp_pairs<T, G>() * sizeof(typename PairOf<T>::P);
}

// resident CTAs per SM the register allocation targets: FP32 in-plane 3 (168
// registers, no spills, with the y-direction carries in shared memory),
// antiplane 5 (96 registers); FP64 in-plane 2, antiplane 4
template <typename T, int G> struct MarchMinBlocks {
  static constexpr int value = sizeof(T) == 4 ? ((G == 0) ? 3 : 5) : ((G == 0) ? 2 : 4);
};

// asynchronous copy of one element into shared memory (completion tracked per
// thread); nbytes = sizeof(T), or 0: nothing is read and zeros are written
template <typename T> TMK_D void cp_async_elem(T* dst_smem, const T* src, unsigned nbytes = sizeof(T)) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst_smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], %2, %3;" ::"r"(d), "l"(src), "n"(sizeof(T)), "r"(nbytes)
               : "memory");
}
TMK_D void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
TMK_D void cp_async_wait_all_but_newest() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }

// The inputs of a cell's plastic return the in-plane group does not hold: the
// antiplane group's updated sxz, syz (stored by the antiplane kernel, which
// has completed) and the plastic strain of the step's input, both sides.
template <typename T>
TMK_D void plastic_inputs(const PatchDev<T>& pp, size_t o, size_t plane, typename PairOf<T>::P* pin) {
  pin[0] = mk2(pp.Uout[o + 7 * plane], pp.Uout[o + 18 * plane]);
  pin[1] = mk2(pp.Uout[o + 8 * plane], pp.Uout[o + 19 * plane]);
  pin[2] = mk2(pp.Uin[o + 10 * plane], pp.Uin[o + 21 * plane]);
}

// Stores the updated group G of one cell (flat index o of component 0).  With
// PL (a plastic level whose return is fused) the in-plane group first takes
// LinElastLevelGodunov::plasticUpdate (PLASTICCORRECTION,
// srcLinElast/PlasticPhysicsF.ChF:30-133, as the reference applies it after
// the level's update, LinElastLevelGodunov.cpp:643-667): the cell's six
// updated stresses and its plastic strain (pin, from plastic_inputs) give the
// return; the antiplane stresses are rewritten where the point yielded, the
// plastic rate and strain always.
template <typename T, int G, bool PL>
TMK_D void store_cell(const PatchDev<T>& pp, const MarchConst<T>& mc, size_t o, size_t plane,
                      typename PairOf<T>::P* u, const typename PairOf<T>::P* pin) {
  constexpr int N = Grp<G>::N;
  if constexpr (G == 0 && PL) {
    T sxz[2] = {pin[0].x, pin[0].y}, syz[2] = {pin[1].x, pin[1].y}, gam[2] = {pin[2].x, pin[2].y};
#pragma unroll
    for (int sd = 0; sd < 2; ++sd) {
      T sxx = sd ? u[2].y : u[2].x, syy = sd ? u[3].y : u[3].x;
      T szz = sd ? u[4].y : u[4].x, sxy = sd ? u[5].y : u[5].x;
      T lam;
      if (plastic_flow_k<T>(mc.pk, sxx, syy, szz, sxy, sxz[sd], syz[sd], lam, gam[sd], mc.pdt)) {
        if (sd) { u[2].y = sxx; u[3].y = syy; u[4].y = szz; u[5].y = sxy; }
        else { u[2].x = sxx; u[3].x = syy; u[4].x = szz; u[5].x = sxy; }
        pp.Uout[o + (size_t)(11 * sd + 7) * plane] = sxz[sd];
        pp.Uout[o + (size_t)(11 * sd + 8) * plane] = syz[sd];
      }
      pp.Uout[o + (size_t)(11 * sd + 9) * plane] = lam;
      pp.Uout[o + (size_t)(11 * sd + 10) * plane] = gam[sd];
    }
  }
#pragma unroll
  for (int c = 0; c < N; ++c) {
    const int gg = Grp<G>::glob(c);
    pp.Uout[o + (size_t)gg * plane] = u[c].x;
    pp.Uout[o + (size_t)(11 + gg) * plane] = u[c].y;
  }
}

// Fluxes of the coarse-fine faces of row `row` that this item owns, into the
// level's flux-register capture buffer (flux registers of the AMR coupling).
// Entry kinds: 0 the x face below the lane's column, 1 the one above, 2 the
// y face below the row, 3 the one above; entries are sorted by row and the
// loop is uniform over the warp.
template <typename T, int G>
TMK_D void march_capture(const PatchDev<T>& pp, const MarchItem& it, const MarchConst<T>& mc, int row, int lane,
                         const typename PairOf<T>::P* Fx, const typename PairOf<T>::P* Fxh,
                         const typename PairOf<T>::P* Fylo, const typename PairOf<T>::P* Fyhi, int& cpos) {
  using P = typename PairOf<T>::P;
  constexpr int N = Grp<G>::N;
  const int4* caps = mc.caps[G];
  const int cend = it.cap0 + it.ncap;
  while (cpos < cend) {
    const int4 e = caps[cpos];
    if (e.x > row) break;
    ++cpos;
    if (e.x < row || e.z != lane) continue;   // rows left to the fault-row kernel, other lanes
#pragma unroll
    for (int c = 0; c < N; ++c) {
      const P v = e.y == 0 ? Fx[c] : e.y == 1 ? Fxh[c] : e.y == 2 ? Fylo[c] : Fyhi[c];
      const int g = Grp<G>::glob(c);
      pp.cap[(size_t)e.w * 22 + g] = (double)v.x;
      pp.cap[(size_t)e.w * 22 + 11 + g] = (double)v.y;
    }
  }
}

// The predictor scheme of every reference deck (PPM, primitive limiting, no
// characteristic limiting), fixed at compile time: SCH = 1.  SCH = 0 reads the
// scheme flags from the launch constants.
constexpr int MARCH_SCH_RUNTIME = 0, MARCH_SCH_PPM_PRIM = 1;
template <typename T>
TMK_HD bool march_scheme_fixed(const MarchConst<T>& mc) { return mc.ppm && mc.plim && !mc.clim; }

// PL: a plastic level with the fused return (in-plane group only): every
// stored cell takes the plastic return, and the kernel runs after the
// antiplane one.
template <typename T, int G, bool PL = false, int SCH = MARCH_SCH_RUNTIME>
__global__ void __launch_bounds__(32 * MARCH_WARPS, MarchMinBlocks<T, G>::value) march_kernel(const PatchDev<T>* __restrict__ patches,
                                                                 const MarchItem* __restrict__ items, int nitems,
                                                                 const __grid_constant__ MarchConst<T> mc) {
  using P = typename PairOf<T>::P;
  constexpr int N = Grp<G>::N;
  extern __shared__ __align__(16) unsigned char march_smem[];
  P* const carry = reinterpret_cast<P*>(march_smem) + (size_t)(threadIdx.x >> 5) * march_warp_pairs<T, G>();
  P* const ring = carry + carry_slots<T, G>() * 32;
  const int wid = blockIdx.x * MARCH_WARPS + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  // a later kernel of the step may be scheduled now; every warp waits for the
  // kernel before it (the fault kernel or the other component group) before
  // it reads the fault buffers or exits, so kernels still complete in order
  asm volatile("griddepcontrol.launch_dependents;");
  if (wid >= nitems) {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    return;
  }
  // the fused plastic return reads the antiplane kernel's stresses: wait for it
  if (PL) asm volatile("griddepcontrol.wait;" ::: "memory");
  const MarchItem it = items[wid];
  const PatchDev<T>& pp = patches[it.patch];
  const int x = it.x0 - MARCH_HALO + lane;
  const int dlo0 = pp.dlo0, dhi0 = pp.dhi0, dlo1 = pp.dlo1, dhi1 = pp.dhi1;
  const int ahi0 = pp.alo0 + pp.anx - 1;
  const bool lane_in = x >= dlo0 && x <= dhi0 && x >= pp.alo0 && x <= ahi0;
  // lane 0 also stages the column left of it (ring entry 0), lane 31 the one
  // right of it (entry 33), each from its own column's address -1 / +1
  const int dxe = lane == 0 ? -1 : 1;
  const bool ext_in = (lane == 0 || lane == 31) && x + dxe >= dlo0 && x + dxe <= dhi0 && x + dxe >= pp.alo0 &&
                      x + dxe <= ahi0;
  const int ext_pos = lane == 0 ? 0 : 33;
  const bool inL = x - 1 >= dlo0, inR = x + 1 <= dhi0;
  constexpr bool kFixed = SCH == MARCH_SCH_PPM_PRIM;
  const bool plim = kFixed || mc.plim != 0, clim = !kFixed && mc.clim != 0, lim = kFixed || mc.lim != 0;
  const bool ppm = kFixed || mc.ppm != 0;
  const MK<T>& kx = mc.kx;
  const MK<T>& ky = mc.ky;
  const P sc = mc.sc;
  const BgView<G, P> bg{mc.bg};
  const bool xout_lo = mc.xout_lo != 0, xout_hi = mc.xout_hi != 0, yout_lo = mc.yout_lo != 0,
             yout_hi = mc.yout_hi != 0;
  const bool fault = pp.fault != 0;
  const bool defer0 = it.fslot >= 0;      // row 0 is finished by march_fault_row_kernel
  const bool col_valid = x >= it.x0 && x < it.x0 + MARCH_COLS && x >= pp.vlo0 && x <= pp.vhi0;
  const size_t plane = (size_t)pp.anx * pp.any;
  // a lane of this warp holds a face on a domain x edge: the x Riemann solves
  // are the interior ones for every lane, overwritten there by the edge
  // condition; other warps (most) skip the edge code on a uniform branch
  const bool warp_xedge = __any_sync(0xffffffffu, x == dlo0 || x == dhi0 + 1);

  auto load_row = [&](int y, P* w) {
    const bool ok = lane_in && y >= dlo1 && y <= dhi1;
    const size_t o = ok ? fab_idx(pp, 0, x, y) : 0;
#pragma unroll
    for (int c = 0; c < N; ++c) {
      const int g = Grp<G>::glob(c);
      w[c] = ok ? mk2(pp.Uin[o + (size_t)g * plane], pp.Uin[o + (size_t)(11 + g) * plane]) : mk2(T(0), T(0));
    }
  };
  // row y into its ring slot: cp.async for cells in the domain, zeros
  // elsewhere; the two outer columns only for the components live in x (the
  // only ones whose neighbours are read)
  auto ring_row = [&](int y) -> P* { return ring + (size_t)((y & (MARCH_RING - 1)) * N) * MARCH_RW; };
  auto load_row_async = [&](int y) {
    const bool yin = y >= dlo1 && y <= dhi1;
    const bool ok = lane_in && yin;
    const size_t o = ok ? fab_idx(pp, 0, x, y) : 0;
    const unsigned nb = ok ? (unsigned)sizeof(T) : 0u;
    P* const rowp = ring_row(y);
    P* const dst = rowp + lane + 1;
    const T* const src = pp.Uin + o;
#pragma unroll
    for (int c = 0; c < N; ++c) {
      const int g = Grp<G>::glob(c);
      T* d2 = reinterpret_cast<T*>(dst + c * MARCH_RW);
      cp_async_elem(d2, src + (size_t)g * plane, nb);
      cp_async_elem(d2 + 1, src + (size_t)(11 + g) * plane, nb);
    }
    if (lane == 0 || lane == 31) {      // the outer columns: own address -1 / +1 (oke implies ok)
      const bool oke = ext_in && yin;
      const unsigned nbe = oke ? (unsigned)sizeof(T) : 0u;
      const T* const srce = oke ? src + dxe : src;
      P* const dste = rowp + ext_pos;
#pragma unroll
      for (int c = 0; c < N; ++c) {
        if (!live<G, 0>(c)) continue;
        const int g = Grp<G>::glob(c);
        T* d2 = reinterpret_cast<T*>(dste + c * MARCH_RW);
        cp_async_elem(d2, srce + (size_t)g * plane, nbe);
        cp_async_elem(d2 + 1, srce + (size_t)(11 + g) * plane, nbe);
      }
    }
    cp_async_commit();
  };
  // the outer columns of row y, loaded directly (the rows staged before the loop)
  auto store_ext_sync = [&](int y) {
    if (lane == 0 || lane == 31) {
      const bool oke = ext_in && y >= dlo1 && y <= dhi1;
      const size_t oe = oke ? fab_idx(pp, 0, x + dxe, y) : 0;
      P* de = ring_row(y) + ext_pos;
#pragma unroll
      for (int c = 0; c < N; ++c) {
        if (!live<G, 0>(c)) continue;
        const int g = Grp<G>::glob(c);
        de[c * MARCH_RW] = oke ? mk2(pp.Uin[oe + (size_t)g * plane], pp.Uin[oe + (size_t)(11 + g) * plane])
                               : mk2(T(0), T(0));
      }
    }
  };
  auto get_row = [&](int y, P* w) {
    const P* src = ring_row(y) + lane + 1;
#pragma unroll
    for (int c = 0; c < N; ++c) w[c] = src[c * MARCH_RW];
  };

  // x-direction normal predictor of row w (its ring row: rw) and the
  // first-pass x-face state on the lane's lo face (H1 lo) and hi face (H1 hi)
  auto xrow = [&](const P* w, const P* rw, P* WM, P* WP, P* H1lo, P* H1hi) {
    if (ppm) {
      P dm[N], dp[N];
#pragma unroll
      for (int c = 0; c < N; ++c) {
        if (!live<G, 0>(c)) { dm[c] = mk2(T(0), T(0)); dp[c] = dm[c]; continue; }
        const P wl = rw[c * MARCH_RW + lane], wr = rw[c * MARCH_RW + lane + 2];
        P s = slope2(wl, w[c], wr, inL, inR, lim);
        P sl = shfl_up2(s, 1);
        P flo = inL ? face2<T>(wl, w[c], sl, s) : pfma(mk2(T(-0.5), T(-0.5)), s, w[c]);
        P fhi = shfl_dn2(flo, 1);
        if (!inR) fhi = pfma(mk2(T(0.5), T(0.5)), s, w[c]);
        dm[c] = psub(flo, w[c]);
        dp[c] = psub(fhi, w[c]);
      }
      predict<G, 0, T>(kx, w, dm, dp, plim, clim, WM, WP);
    } else {
#pragma unroll
      for (int c = 0; c < N; ++c) { WM[c] = w[c]; WP[c] = w[c]; }
    }
    P L[N];
#pragma unroll
    for (int c = 0; c < N; ++c) L[c] = live<G, 0>(c) ? shfl_up2(WP[c], 1) : mk2(T(0), T(0));
    riem<G, 0, T>(kx, L, WM, H1lo);
    if (warp_xedge) {                 // the domain-edge conditions, only in warps that reach an x edge
      if (x == dlo0) edge2<G, 0, T>(kx, true, xout_lo, WM, bg, H1lo);
      else if (x == dhi0 + 1) edge2<G, 0, T>(kx, false, xout_hi, L, bg, H1lo);
    }
#pragma unroll
    for (int c = 0; c < N; ++c) H1hi[c] = live<G, 0>(c) ? shfl_dn2(H1lo[c], 1) : mk2(T(0), T(0));
  };

  const int q_s = max(it.y0 - 1, dlo1);
  const int q_e = it.y1 + 1;
  int cpos = it.cap0;                     // next coarse-fine face to store
  P rcar[kNumCarry - kWPy][N];     // the register-resident carries (FP64 form)
  auto cput = [&](int v, const P* a) {
#pragma unroll
    for (int c = 0; c < N; ++c) {
      if (!carry_needed<G>(v, c)) continue;
      if (carry_in_smem<T>(v)) carry[carry_slot<T, G>(v, c) * 32 + lane] = a[c];
      else rcar[v - kWPy][c] = a[c];
    }
  };
  auto cget = [&](int v, P* a) {
#pragma unroll
    for (int c = 0; c < N; ++c)
      a[c] = !carry_needed<G>(v, c) ? mk2(T(0), T(0))
             : carry_in_smem<T>(v) ? carry[carry_slot<T, G>(v, c) * 32 + lane] : rcar[v - kWPy][c];
  };
  // rolling window of rows q, q+1, q+2 (ring slots); slope(q) and the lo-face value of row q carried
  {
    P Wa[N], Wb[N], W0[N], W1[N], W2[N], sy0[N], Fy0[N];
    load_row(q_s - 2, Wa);
    load_row(q_s - 1, Wb);
    load_row(q_s, W0);
    load_row(q_s + 1, W1);
    load_row(q_s + 2, W2);
    {
      P* r0 = ring_row(q_s) + lane + 1; P* r1 = ring_row(q_s + 1) + lane + 1; P* r2 = ring_row(q_s + 2) + lane + 1;
#pragma unroll
      for (int c = 0; c < N; ++c) { r0[c * MARCH_RW] = W0[c]; r1[c * MARCH_RW] = W1[c]; r2[c * MARCH_RW] = W2[c]; }
      store_ext_sync(q_s);
      store_ext_sync(q_s + 1);
      store_ext_sync(q_s + 2);
    }
    const bool hl = q_s - 1 >= dlo1, hr = q_s + 1 <= dhi1;
#pragma unroll
    for (int c = 0; c < N; ++c) {
      if (!live<G, 1>(c)) { sy0[c] = mk2(T(0), T(0)); Fy0[c] = sy0[c]; continue; }
      sy0[c] = slope2(Wb[c], W0[c], W1[c], hl, hr, lim);
      if (hl) {
        P sm = slope2(Wa[c], Wb[c], W0[c], q_s - 2 >= dlo1, true, lim);
        Fy0[c] = face2<T>(Wb[c], W0[c], sm, sy0[c]);
      } else {
        Fy0[c] = pfma(mk2(T(-0.5), T(-0.5)), sy0[c], W0[c]);
      }
    }
    cput(kSy, sy0);
    cput(kFyf, Fy0);
  }

  for (int q = q_s; q <= q_e; ++q) {
    const bool rowin = q <= dhi1;
    load_row_async(q + 3);            // next row in flight while this one is computed
    // fused plastic return: its other inputs for row q-1, stored at the end of
    // this iteration, requested now so that the row's work hides their latency
    P pin[3];
    if constexpr (PL) {
      if (col_valid && q - 1 >= it.y0 && q - 1 <= it.y1) plastic_inputs<T>(pp, fab_idx(pp, 0, x, q - 1), plane, pin);
    }
    cp_async_wait_all_but_newest();   // rows up to q+2 have landed
    __syncwarp();                     // ... every lane's copies, whose neighbours read them
    P W0[N], W1[N], W2[N];
    get_row(q, W0);
    get_row(q + 1, W1);
    get_row(q + 2, W2);
    P WMy[N], WPy[N], WMcy[N], WPcy[N], WMx[N], WPx[N], H1lo[N], H1hi[N];
    P sy1[N], Fy1[N];
    if (rowin) {
      // y predictor of row q
      if (ppm) {
        const bool hl = true, hr = q + 2 <= dhi1;
        P dm[N], dp[N], sy0[N], Fy0[N];
        cget(kSy, sy0);
        cget(kFyf, Fy0);
#pragma unroll
        for (int c = 0; c < N; ++c) {
          if (!live<G, 1>(c)) { sy1[c] = mk2(T(0), T(0)); Fy1[c] = sy1[c]; dm[c] = sy1[c]; dp[c] = sy1[c]; continue; }
          sy1[c] = slope2(W0[c], W1[c], W2[c], hl, hr, lim);
          Fy1[c] = (q + 1 <= dhi1) ? face2<T>(W0[c], W1[c], sy0[c], sy1[c])
                                   : pfma(mk2(T(0.5), T(0.5)), sy0[c], W0[c]);
          dm[c] = psub(Fy0[c], W0[c]);
          dp[c] = psub(Fy1[c], W0[c]);
        }
        predict<G, 1, T>(ky, W0, dm, dp, plim, clim, WMy, WPy);
        cput(kSy, sy1);
        cput(kFyf, Fy1);
      } else {
#pragma unroll
        for (int c = 0; c < N; ++c) { WMy[c] = W0[c]; WPy[c] = W0[c]; }
      }
      // x predictor of row q, first-pass x faces, corrected y states of row q
      xrow(W0, ring_row(q), WMx, WPx, H1lo, H1hi);
#pragma unroll
      for (int c = 0; c < N; ++c) { WMcy[c] = WMy[c]; WPcy[c] = WPy[c]; }
      adw2<G, 0, T>(kx, H1hi, H1lo, WMcy, WPcy);
    }
    // first-pass y face q (lo face of row q)
    P H1y[N];
    P WPy_p[N];
    cget(kWPy, WPy_p);
    const bool need_h1y = (q > q_s) || (q == dlo1);
    if (need_h1y) {
      if (q == dlo1) {
        if (fault) {
          // the fault kernel's first-pass face state: only row 0's transverse
          // correction reads it, and row 0 of a fault patch is finished later
#pragma unroll
          for (int c = 0; c < N; ++c) H1y[c] = mk2(T(0), T(0));
        } else {
          edge2<G, 1, T>(ky, true, yout_lo, WMy, bg, H1y);
        }
      } else if (!rowin) {
        edge2<G, 1, T>(ky, false, yout_hi, WPy_p, bg, H1y);
      } else {
        riem<G, 1, T>(ky, WPy_p, WMy, H1y);
      }
    }
    // final y face q
    P Fy[N];
    P WPcy_p[N];
    cget(kWPcy, WPcy_p);
    if (q >= it.y0) {
      if (q == dlo1 && fault) {
#pragma unroll
        for (int c = 0; c < N; ++c) Fy[c] = mk2(T(0), T(0));   // the fault flux: row 0 is finished later
      } else {
        P g[N];
        if (q == dlo1) edge2<G, 1, T>(ky, true, yout_lo, WMcy, bg, g);
        else if (!rowin) edge2<G, 1, T>(ky, false, yout_hi, WPcy_p, bg, g);
        else riem<G, 1, T>(ky, WPcy_p, WMcy, g);
        flux2<G, 1, T>(ky, g, Fy);
      }
    }
    // row q-1: transverse correction of its x states, final x faces, update;
    // row 0 of a fault patch: keep what march_fault_row_kernel needs
    if (defer0 && q - 1 == dlo1) {
      P* st = reinterpret_cast<P*>(mc.stash[G]) + (size_t)it.fslot * MARCH_STASH_VECS * N * 32 + lane;
      P a[N];
      cget(kWMx, a);
#pragma unroll
      for (int c = 0; c < N; ++c) st[(0 * N + c) * 32] = a[c];
      cget(kWPx, a);
#pragma unroll
      for (int c = 0; c < N; ++c) st[(1 * N + c) * 32] = a[c];
#pragma unroll
      for (int c = 0; c < N; ++c) { st[(2 * N + c) * 32] = H1y[c]; st[(3 * N + c) * 32] = Fy[c]; }
      cget(kWold, a);
#pragma unroll
      for (int c = 0; c < N; ++c) st[(4 * N + c) * 32] = a[c];
    } else if (q - 1 >= it.y0) {
      P WMcx[N], WPcx[N];
      {
        P H1y_p[N];
        cget(kWMx, WMcx);
        cget(kWPx, WPcx);
        cget(kH1y, H1y_p);
        adw2<G, 1, T>(ky, H1y, H1y_p, WMcx, WPcx);
      }
      P L[N], g[N], Fx[N], Fxh[N];
#pragma unroll
      for (int c = 0; c < N; ++c) L[c] = live<G, 0>(c) ? shfl_up2(WPcx[c], 1) : mk2(T(0), T(0));
      riem<G, 0, T>(kx, L, WMcx, g);
      if (warp_xedge) {
        if (x == dlo0) edge2<G, 0, T>(kx, true, xout_lo, WMcx, bg, g);
        else if (x == dhi0 + 1) edge2<G, 0, T>(kx, false, xout_hi, L, bg, g);
      }
      flux2<G, 0, T>(kx, g, Fx);
#pragma unroll
      for (int c = 0; c < N; ++c) Fxh[c] = shfl_dn2(Fx[c], 1);
      const int yr = q - 1;
      P Fy_p[N], Wold[N];
      cget(kFy, Fy_p);
      cget(kWold, Wold);
      if (col_valid && yr <= it.y1) {
        P u[N];
#pragma unroll
        for (int c = 0; c < N; ++c) u[c] = pfma(padd(psub(Fxh[c], Fx[c]), psub(Fy[c], Fy_p[c])), sc, Wold[c]);
        store_cell<T, G, PL>(pp, mc, fab_idx(pp, 0, x, yr), plane, u, pin);
      }
      if (it.ncap && yr <= it.y1) march_capture<T, G>(pp, it, mc, yr, lane, Fx, Fxh, Fy_p, Fy, cpos);
    }
    // advance the window
    cput(kWMx, WMx);
    cput(kWPx, WPx);
    cput(kH1y, H1y);
    cput(kFy, Fy);
    cput(kWold, W0);
    cput(kWPy, WPy);
    cput(kWPcy, WPcy);
  }
  asm volatile("cp.async.wait_all;" ::: "memory");
  asm volatile("griddepcontrol.wait;" ::: "memory");
}

// Row 0 of a fault-row strip of group G once the fault kernel has produced the
// first-pass fault states and the fault-face fluxes: the transverse correction
// of the row's x states, its final x faces and its update (the same steps as
// the marching loop, with the stashed row-0 intermediates).
template <typename T, int G>
TMK_D void fault_row_finish(const PatchDev<T>& pp, const MarchItem& it, const MarchConst<T>& mc, int lane) {
  using P = typename PairOf<T>::P;
  constexpr int N = Grp<G>::N;
  const int x = it.x0 - MARCH_HALO + lane;
  const int dlo0 = pp.dlo0, dhi0 = pp.dhi0, dlo1 = pp.dlo1;
  const P* st = reinterpret_cast<const P*>(mc.stash[G]) + (size_t)it.fslot * MARCH_STASH_VECS * N * 32 + lane;
  P WMcx[N], WPcx[N], H1y1[N], Fy1[N], Wold[N], H1y0[N], Fy0[N];
#pragma unroll
  for (int c = 0; c < N; ++c) {
    WMcx[c] = st[(0 * N + c) * 32]; WPcx[c] = st[(1 * N + c) * 32];
    H1y1[c] = st[(2 * N + c) * 32]; Fy1[c] = st[(3 * N + c) * 32]; Wold[c] = st[(4 * N + c) * 32];
  }
  const int fi1 = x - (pp.vlo0 - 1);
  const bool ok1 = fi1 >= 0 && fi1 < pp.nfirst && x >= dlo0 && x <= dhi0;
  const int nv = pp.vhi0 - pp.vlo0 + 1, fi2 = x - pp.vlo0;
  const bool ok2 = fi2 >= 0 && fi2 < nv;
#pragma unroll
  for (int c = 0; c < N; ++c) {
    const int g = Grp<G>::glob(c);
    H1y0[c] = ok1 ? mk2((T)pp.first[(size_t)g * pp.nfirst + fi1], (T)pp.first[(size_t)(11 + g) * pp.nfirst + fi1])
                  : mk2(T(0), T(0));
    Fy0[c] = ok2 ? mk2((T)pp.ffault[(size_t)g * nv + fi2], (T)pp.ffault[(size_t)(11 + g) * nv + fi2])
                 : mk2(T(0), T(0));
  }
  adw2<G, 1, T>(mc.ky, H1y1, H1y0, WMcx, WPcx);
  const BgView<G, P> bg{mc.bg};
  P L[N], g[N], Fx[N], Fxh[N];
#pragma unroll
  for (int c = 0; c < N; ++c) L[c] = live<G, 0>(c) ? shfl_up2(WPcx[c], 1) : mk2(T(0), T(0));
  if (x == dlo0) edge2<G, 0, T>(mc.kx, true, mc.xout_lo != 0, WMcx, bg, g);
  else if (x == dhi0 + 1) edge2<G, 0, T>(mc.kx, false, mc.xout_hi != 0, L, bg, g);
  else riem<G, 0, T>(mc.kx, L, WMcx, g);
  flux2<G, 0, T>(mc.kx, g, Fx);
#pragma unroll
  for (int c = 0; c < N; ++c) Fxh[c] = shfl_dn2(Fx[c], 1);
  if (it.ncap) {
    int cpos = it.cap0;
    march_capture<T, G>(pp, it, mc, dlo1, lane, Fx, Fxh, Fy0, Fy1, cpos);
  }
  const bool col_valid = x >= it.x0 && x < it.x0 + MARCH_COLS && x >= pp.vlo0 && x <= pp.vhi0;
  if (col_valid) {
    P u[N];
#pragma unroll
    for (int c = 0; c < N; ++c) u[c] = pfma(padd(psub(Fxh[c], Fx[c]), psub(Fy1[c], Fy0[c])), mc.sc, Wold[c]);
    const size_t plane = (size_t)pp.anx * pp.any, o = fab_idx(pp, 0, x, dlo1);
    P pin[3];
    if (mc.plastic) {
      plastic_inputs<T>(pp, o, plane, pin);
      store_cell<T, G, true>(pp, mc, o, plane, u, pin);
    } else {
      store_cell<T, G, false>(pp, mc, o, plane, u, pin);
    }
  }
}

// One warp per fault-row strip: rows0 (in-plane) then rows1 (antiplane).  With
// the fused plastic return the antiplane rows are finished by a launch of
// their own before the in-plane ones (whose stores apply the return).
template <typename T>
__global__ void __launch_bounds__(32 * MARCH_WARPS) march_fault_row_kernel(const PatchDev<T>* __restrict__ patches,
                                                                           const MarchItem* __restrict__ rows0, int n0,
                                                                           const MarchItem* __restrict__ rows1, int n1,
                                                                           const __grid_constant__ MarchConst<T> mc) {
  const int wid = blockIdx.x * MARCH_WARPS + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (wid < n0) {
    const MarchItem it = rows0[wid];
    fault_row_finish<T, 0>(patches[it.patch], it, mc, lane);
  } else if (wid < n0 + n1) {
    const MarchItem it = rows1[wid - n0];
    fault_row_finish<T, 1>(patches[it.patch], it, mc, lane);
  }
}

#undef KC
#undef KE
#undef KHALF

}  // namespace tmk
