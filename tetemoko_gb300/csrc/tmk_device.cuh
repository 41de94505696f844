// tmk_device.cuh -- per-point physics of the GB300 Godunov step.
//
// Every routine works on ONE side of the fault (9 state components, local order
// vx vy vz sxx syy szz sxy sxz syz) in ONE direction D (0 = x, 1 = y).  The two
// sides of the mirrored grid only meet at the fault face, and inside the
// volume the reference's 22-component transforms are block-diagonal by side,
// so the volume kernel runs one side per CTA.
//
// Two arithmetic policies share the code:
//   * double: the reference's operation order (srcLinElast/LinElastPhysicsF.ChF),
//     compiled without FMA contraction, so the FP64 path matches the CPU oracle
//     to rounding;
//   * float : the same formulas with divisions replaced by precomputed
//     reciprocals, for the mixed-precision volume kernel.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <type_traits>

#define TMK_HD __host__ __device__ __forceinline__
#define TMK_D __device__ __forceinline__

namespace tmk {

constexpr int NC = 22;
constexpr int NSIDE = 9;          // evolving components per side
constexpr int NGHOST = 4;
constexpr int SW_MAXP = 8;

// Per-scenario parameters (the reference's COMMON blocks, precomputed on the host).
struct DevParams {
  // /IBC/ (LINELASTSETF)
  double cs, cp, G, rho, lam, K, Zp, Zs;
  double bg[22];
  // scheme
  int order, prim_lim, char_lim;
  int fourth;               // fourth-order slopes (PLM)
  int bc[6];
  int fault_law;            // 0 none, 1 RS, 2 SW
  int plasticity;
  // rate and state (RSSETF)
  double rs_r0, rs_x0, rs_nsig, rs_a, rs_b, rs_V0, rs_f0, rs_L, rs_fw, rs_Vw, rs_fexp;
  double ramp_x, ramp_w, ramp_a, ramp_Vw, rs_thr;
  int state_law;
  // slip weakening (SWSETF + SWIBC members)
  double sw_fs, sw_fd, sw_dw, sw_smooth;
  int sw_np;
  double sw_xc[SW_MAXP], sw_xw[SW_MAXP], sw_tau[SW_MAXP];
  double sw_fbc0, sw_fbw0, sw_outside, sw_thr;
  int sw_off;               // side-2 component offset, 9 (reference) or 11
  double sw_zc[SW_MAXP], sw_zw[SW_MAXP], sw_fbc1, sw_fbw1;   // z profiles (3-D)
  // plasticity (PLASTICSETF)
  double p_mu, p_beta, p_eta, p_b, p_h;
  // reciprocals the mixed form's friction solve multiplies by (its chain of
  // FP64 operations is the fault kernel's latency; a division costs several)
  double inv_Zs, inv_Zp, lam_r, two_V0, inv_2V0;   // lam_r = lam/(lam+2G)
  double ln_2V0, ln_halfZs;                          // log(2 V0), log(Zs / 2)
};

// Constants of one arithmetic type.
template <typename T>
struct Consts {
  T lam, G, rho, Zp, Zs, lam2G;           // lam2G = 2G + lam
  T inv_rho, inv_Zp, inv_Zs, ratio;       // ratio = lam/(2G+lam)
  T half_inv_Zp, half_inv_Zs, lamp2G;     // lamp2G = lam + 2G
  T cs, cp;
  TMK_HD void load(const DevParams& p) {
    lam = (T)p.lam; G = (T)p.G; rho = (T)p.rho; Zp = (T)p.Zp; Zs = (T)p.Zs;
    lam2G = (T)(2.0 * p.G + p.lam);
    lamp2G = (T)(p.lam + 2.0 * p.G);
    inv_rho = (T)(1.0 / p.rho); inv_Zp = (T)(1.0 / p.Zp); inv_Zs = (T)(1.0 / p.Zs);
    ratio = (T)(p.lam / (2.0 * p.G + p.lam));
    half_inv_Zp = (T)(0.5 / p.Zp); half_inv_Zs = (T)(0.5 / p.Zs);
    cs = (T)p.cs; cp = (T)p.cp;
  }
};

template <typename T> constexpr bool kExact = std::is_same<T, double>::value;

// Rotation of LinElastPhysicsF.ChF's directional routines (cx, cy, cz, cxy, cxz, cyz).
template <int D> struct Rot;
template <> struct Rot<0> { static constexpr int cx = 0, cy = 1, cz = 2, cxy = 6, cxz = 7, cyz = 8; };
template <> struct Rot<1> { static constexpr int cx = 1, cy = 2, cz = 0, cxy = 8, cxz = 6, cyz = 7; };
template <> struct Rot<2> { static constexpr int cx = 2, cy = 0, cz = 1, cxy = 7, cxz = 8, cyz = 6; };

// Components of one side's state in direction D that a face state's flux and
// transverse term never read: the zero-speed ones (cy+3, cz+3, cyz).  RIEMANNF
// and the edge conditions form the components the fluxes read (cx, cy, cz,
// cx+3, cxy, cxz) from the same components of the states they are given.
template <int D> TMK_HD constexpr bool live9(int c) {
  using R = Rot<D>;
  return c != R::cy + 3 && c != R::cz + 3 && c != R::cyz;
}

// lambda-ratio product  s*lam/(2G+lam)
template <typename T> TMK_D T lratio(const Consts<T>& k, T s) {
  if constexpr (kExact<T>) return s * k.lam / k.lam2G; else return s * k.ratio;
}

// ---------------------------------------------------------------- CHARANALYSISF
// Output order of the nine characteristic variables of one side:
//   0 sxx+Zp vx (-cp)  1 sxy+Zs vy (-cs)  2 sxz+Zs vz (-cs)  3 wyy (0)  4 wzz (0)
//   5 wyz (0)  6 sxz-Zs vz (+cs)  7 sxy-Zs vy (+cs)  8 sxx-Zp vx (+cp)
template <int D, typename T>
TMK_D void char_analysis(const Consts<T>& k, T rv, const T* q, T* w) {
  using R = Rot<D>;
  T vx = rv * q[R::cx], vy = rv * q[R::cy], vz = rv * q[R::cz];
  T sxx = q[R::cx + 3], syy = q[R::cy + 3], szz = q[R::cz + 3];
  T sxy = q[R::cxy], sxz = q[R::cxz], syz = q[R::cyz];
  w[0] = sxx + vx * k.Zp;
  w[1] = sxy + vy * k.Zs;
  w[2] = sxz + vz * k.Zs;
  w[3] = syy - lratio(k, sxx);
  w[4] = szz - lratio(k, sxx);
  w[5] = syz;
  w[6] = sxz - vz * k.Zs;
  w[7] = sxy - vy * k.Zs;
  w[8] = sxx - vx * k.Zp;
}

// ---------------------------------------------------------------- CHARSYNTHESISF
template <int D, typename T>
TMK_D void char_synthesis(const Consts<T>& k, T rv, const T* w, T* q) {
  using R = Rot<D>;
  T wxxm = w[0], wxym = w[1], wxzm = w[2], wyy = w[3], wzz = w[4], wyz = w[5];
  T wxzp = w[6], wxyp = w[7], wxxp = w[8];
  T sxx = (wxxm + wxxp) / T(2);
  if constexpr (kExact<T>) {
    q[R::cx] = rv * (wxxm - wxxp) / 2.0 / k.Zp;
    q[R::cy] = rv * (wxym - wxyp) / 2.0 / k.Zs;
    q[R::cz] = rv * (wxzm - wxzp) / 2.0 / k.Zs;
  } else {
    q[R::cx] = rv * (wxxm - wxxp) * k.half_inv_Zp;
    q[R::cy] = rv * (wxym - wxyp) * k.half_inv_Zs;
    q[R::cz] = rv * (wxzm - wxzp) * k.half_inv_Zs;
  }
  q[R::cx + 3] = sxx;
  q[R::cy + 3] = wyy + lratio(k, sxx);
  q[R::cz + 3] = wzz + lratio(k, sxx);
  q[R::cxy] = (wxym + wxyp) / T(2);
  q[R::cxz] = (wxzm + wxzp) / T(2);
  q[R::cyz] = wyz;
}

// ---------------------------------------------------------------- RIEMANNF
template <int D, typename T>
TMK_D void riemann(const Consts<T>& k, T rv, const T* L, const T* Rr, T* g) {
  using R = Rot<D>;
  T wxxp = L[R::cx + 3] - rv * k.Zp * L[R::cx];
  T wxyp = L[R::cxy] - rv * k.Zs * L[R::cy];
  T wxzp = L[R::cxz] - rv * k.Zs * L[R::cz];
  T wxxm = Rr[R::cx + 3] + rv * k.Zp * Rr[R::cx];
  T wxym = Rr[R::cxy] + rv * k.Zs * Rr[R::cy];
  T wxzm = Rr[R::cxz] + rv * k.Zs * Rr[R::cz];
  T wyy = Rr[R::cy + 3] - lratio(k, Rr[R::cx + 3]);
  T wzz = Rr[R::cz + 3] - lratio(k, Rr[R::cx + 3]);
  T wyz = Rr[R::cyz];
  wyy = (wyy + L[R::cy + 3] - lratio(k, L[R::cx + 3])) / T(2);
  wzz = (wzz + L[R::cz + 3] - lratio(k, L[R::cx + 3])) / T(2);
  wyz = (wyz + L[R::cyz]) / T(2);
  T sxx = (wxxm + wxxp) / T(2);
  if constexpr (kExact<T>) {
    g[R::cx] = rv * (wxxm - wxxp) / 2.0 / k.Zp;
    g[R::cy] = rv * (wxym - wxyp) / 2.0 / k.Zs;
    g[R::cz] = rv * (wxzm - wxzp) / 2.0 / k.Zs;
  } else {
    g[R::cx] = rv * (wxxm - wxxp) * k.half_inv_Zp;
    g[R::cy] = rv * (wxym - wxyp) * k.half_inv_Zs;
    g[R::cz] = rv * (wxzm - wxzp) * k.half_inv_Zs;
  }
  g[R::cx + 3] = (wxxm + wxxp) / T(2);
  g[R::cy + 3] = wyy + lratio(k, sxx);
  g[R::cz + 3] = wzz + lratio(k, sxx);
  g[R::cxy] = (wxym + wxyp) / T(2);
  g[R::cxz] = (wxzm + wxzp) / T(2);
  g[R::cyz] = wyz;
}

// ---------------------------------------------------------------- GETFLUXF
template <int D, typename T>
TMK_D void flux(const Consts<T>& k, T rv, const T* g, T* F) {
  using R = Rot<D>;
  T vx = g[R::cx], vy = g[R::cy], vz = g[R::cz];
  T sxx = g[R::cx + 3], sxy = g[R::cxy], sxz = g[R::cxz];
  if constexpr (kExact<T>) {
    F[R::cx] = -rv * sxx / k.rho;
    F[R::cy] = -rv * sxy / k.rho;
    F[R::cz] = -rv * sxz / k.rho;
    F[R::cx + 3] = -rv * vx * (k.lam + 2.0 * k.G);
    F[R::cy + 3] = -rv * vx * k.lam;
    F[R::cz + 3] = -rv * vx * k.lam;
    F[R::cxy] = -rv * vy * k.G;
    F[R::cxz] = -rv * vz * k.G;
  } else {
    T m = -rv;
    F[R::cx] = m * sxx * k.inv_rho;
    F[R::cy] = m * sxy * k.inv_rho;
    F[R::cz] = m * sxz * k.inv_rho;
    F[R::cx + 3] = m * vx * k.lamp2G;
    F[R::cy + 3] = m * vx * k.lam;
    F[R::cz + 3] = m * vx * k.lam;
    F[R::cxy] = m * vy * k.G;
    F[R::cxz] = m * vz * k.G;
  }
  F[R::cyz] = T(0);
}

// ---------------------------------------------------------------- GETADWDXF
// increment of one cell from the face states at its hi (h) and lo (l) faces
template <int D, typename T>
TMK_D void adwdx_add(const Consts<T>& k, T rv, T scale, const T* h, const T* l, T* q) {
  using R = Rot<D>;
  T vx = h[R::cx] - l[R::cx];
  T vy = h[R::cy] - l[R::cy];
  T vz = h[R::cz] - l[R::cz];
  T sxx = h[R::cx + 3] - l[R::cx + 3];
  T sxy = h[R::cxy] - l[R::cxy];
  T sxz = h[R::cxz] - l[R::cxz];
  if constexpr (kExact<T>) {
    q[R::cx] += -rv * scale * sxx / k.rho;
    q[R::cy] += -rv * scale * sxy / k.rho;
    q[R::cz] += -rv * scale * sxz / k.rho;
    q[R::cx + 3] += -rv * scale * vx * (k.lam + 2.0 * k.G);
    q[R::cy + 3] += -rv * scale * vx * k.lam;
    q[R::cz + 3] += -rv * scale * vx * k.lam;
    q[R::cxy] += -rv * scale * vy * k.G;
    q[R::cxz] += -rv * scale * vz * k.G;
    q[R::cyz] += -rv * scale * 0.0;
  } else {
    T m = -rv * scale;
    q[R::cx] += m * sxx * k.inv_rho;
    q[R::cy] += m * sxy * k.inv_rho;
    q[R::cz] += m * sxz * k.inv_rho;
    q[R::cx + 3] += m * vx * k.lamp2G;
    q[R::cy + 3] += m * vx * k.lam;
    q[R::cz + 3] += m * vx * k.lam;
    q[R::cxy] += m * vy * k.G;
    q[R::cxz] += m * vz * k.G;
  }
}

// ------------------------------------------- LINELASTOUTBCF / LINELASTFREEBCF
// Boundary Riemann state of one side at a domain edge.  `bg` is the side's
// background (outflow only).  SHF is the normal VELOCITY minus sxx, as written
// in the reference; it only reaches components no flux or transverse term reads.
template <int D, typename T>
TMK_D void edge_bc(const Consts<T>& k, T rv, int lohisign, bool outflow, const T* bg, const T* wi, T* g) {
  using R = Rot<D>;
  T wpx, wpy, wpz, wmx, wmy, wmz;
  if (outflow) {
    wpx = bg[R::cx + 3] - rv * k.Zp * bg[R::cx];
    wpy = bg[R::cxy] - rv * k.Zs * bg[R::cy];
    wpz = bg[R::cxz] - rv * k.Zs * bg[R::cz];
    wmx = bg[R::cx + 3] + rv * k.Zp * bg[R::cx];
    wmy = bg[R::cxy] + rv * k.Zs * bg[R::cy];
    wmz = bg[R::cxz] + rv * k.Zs * bg[R::cz];
    if (lohisign == -1) {
      wmx = (wi[R::cx + 3] + rv * k.Zp * wi[R::cx]);
      wmy = (wi[R::cxy] + rv * k.Zs * wi[R::cy]);
      wmz = (wi[R::cxz] + rv * k.Zs * wi[R::cz]);
    } else {
      wpx = (wi[R::cx + 3] - rv * k.Zp * wi[R::cx]);
      wpy = (wi[R::cxy] - rv * k.Zs * wi[R::cy]);
      wpz = (wi[R::cxz] - rv * k.Zs * wi[R::cz]);
    }
  } else {
    if (lohisign == -1) {
      wmx = (wi[R::cx + 3] + rv * k.Zp * wi[R::cx]);
      wmy = (wi[R::cxy] + rv * k.Zs * wi[R::cy]);
      wmz = (wi[R::cxz] + rv * k.Zs * wi[R::cz]);
      wpx = -wmx; wpy = -wmy; wpz = -wmz;
    } else {
      wpx = (wi[R::cx + 3] - rv * k.Zp * wi[R::cx]);
      wpy = (wi[R::cxy] - rv * k.Zs * wi[R::cy]);
      wpz = (wi[R::cxz] - rv * k.Zs * wi[R::cz]);
      wmx = -wpx; wmy = -wpy; wmz = -wpz;
    }
  }
  T sxx = (wmx + wpx) / T(2);
  T SHF;
  if constexpr (kExact<T>) {
    SHF = -(wi[R::cx] - sxx) * k.lam / (k.lam + 2.0 * k.G);
    g[R::cx] = rv * (wmx - wpx) / (2.0 * k.Zp);
    g[R::cy] = rv * (wmy - wpy) / (2.0 * k.Zs);
    g[R::cz] = rv * (wmz - wpz) / (2.0 * k.Zs);
  } else {
    SHF = -(wi[R::cx] - sxx) * k.ratio;
    g[R::cx] = rv * (wmx - wpx) * k.half_inv_Zp;
    g[R::cy] = rv * (wmy - wpy) * k.half_inv_Zs;
    g[R::cz] = rv * (wmz - wpz) * k.half_inv_Zs;
  }
  g[R::cx + 3] = sxx;
  g[R::cy + 3] = wi[R::cy + 3] + SHF;
  g[R::cz + 3] = wi[R::cz + 3] + SHF;
  g[R::cxy] = (wmy + wpy) / T(2);
  g[R::cxz] = (wmz + wpz) / T(2);
  g[R::cyz] = wi[R::cyz];
}

// ---------------------------------------------------------------- PPM stages
// Van Leer limited slope of the middle value (one-sided where a neighbour is
// outside the domain).
template <typename T>
TMK_D T vl_slope(T wm, T w0, T wp, bool hasL, bool hasR, bool limit) {
  T dwl, dwr, dwc;
  if (hasL && hasR) {
    dwl = w0 - wm; dwr = wp - w0; dwc = T(0.5) * (wp - wm);
  } else if (hasR) {
    dwr = wp - w0; dwl = dwr; dwc = dwr;
  } else if (hasL) {
    dwl = w0 - wm; dwr = dwl; dwc = dwl;
  } else {
    return T(0);
  }
  if (!limit) return dwc;
  if (dwl * dwr > T(0)) {
    T m = fmin(fabs(dwc), fmin(T(2) * fabs(dwl), T(2) * fabs(dwr)));
    return dwc >= T(0) ? m : -m;
  }
  return T(0);
}

// Face deltas (W_{lo face} - W, W_{hi face} - W) of the PPM parabola of the
// middle cell from five values w[0..4] (cells -2..+2) with in[k] telling
// whether cell k-2 lies in the domain (in[2] is always true).
template <typename T>
TMK_D void ppm_deltas(const T* w, const bool* in, bool limit, T& dm, T& dp) {
  T sm = in[1] ? vl_slope(w[0], w[1], w[2], in[0], true, limit) : T(0);
  T s0 = vl_slope(w[1], w[2], w[3], in[1], in[3], limit);
  T sp = in[3] ? vl_slope(w[2], w[3], w[4], true, in[4], limit) : T(0);
  T flo, fhi;
  if (in[1]) flo = T(0.5) * (w[1] + w[2]) - (s0 - sm) / T(6);
  else       flo = w[2] - T(0.5) * s0;
  if (in[3]) fhi = T(0.5) * (w[2] + w[3]) - (sp - s0) / T(6);
  else       fhi = w[2] + T(0.5) * s0;
  dm = (T(0) - w[2]) + flo;
  dp = (T(0) - w[2]) + fhi;
}

// PPM limiter (Colella & Woodward 1984 eq. 1.10) on one pair of deltas
template <typename T>
TMK_D void ppm_limit(T& m, T& p) {
  if (m * p < T(0)) {
    T am = fmin(fabs(m), T(2) * fabs(p));
    T ap = fmin(fabs(p), T(2) * fabs(m));
    m = m >= T(0) ? am : -am;
    p = p >= T(0) ? ap : -ap;
  } else {
    m = T(0); p = T(0);
  }
}

// PPM characteristic tracing (Colella & Woodward 1984 eq. 1.12) of one
// characteristic with Courant number sig = lambda dt/dx
template <typename T>
TMK_D void ppm_trace(T sig, T& m, T& p) {
  if (sig > T(0)) {
    T s = sig;
    p = p - T(0.5) * s * ((p - m) + T(3) * (T(1) - (T(2) / T(3)) * s) * (m + p));
  } else if (sig < T(0)) {
    T s = -sig;
    m = m + T(0.5) * s * (p - m) - T(3) * (m + p) * (T(0.5) * s - s * s / T(3));
  }
}

// PLM stages (LinElastPatchGodunov::PLMNormalPred, srcLinElast/
// LinElastPatchGodunov.cpp:486-601, with Chombo's slope utilities restated):
// the slope of the middle cell of w[0..4] -- van Leer, or where both
// neighbours lie in the domain and `fourth` is set the fourth-order slope
// (4/3) dWc - (1/6)(dWvL_{+1} + dWvL_{-1}) (Colella & Glaz 1985) --, its
// one-sided differences (the missing one next to a domain edge takes the
// other's value) and the van Leer limiter of a slope by them.
template <typename T>
TMK_D T plm_slope(const T* w, const bool* in, bool limit, bool fourth) {
  const T s0 = vl_slope(w[1], w[2], w[3], in[1], in[3], limit);
  if (!fourth || !in[1] || !in[3]) return s0;
  const T sm = vl_slope(w[0], w[1], w[2], in[0], true, limit);
  const T sp = vl_slope(w[2], w[3], w[4], true, in[4], limit);
  const T dwc = T(0.5) * (w[3] - w[1]);
  return (T(4) / T(3)) * dwc - (T(1) / T(6)) * (sp + sm);
}
template <typename T>
TMK_D void plm_onesided(const T* w, const bool* in, T& m, T& p) {
  m = in[1] ? w[2] - w[1] : T(0);
  p = in[3] ? w[3] - w[2] : T(0);
  if (!in[1]) m = p;
  if (!in[3]) p = m;
}
template <typename T>
TMK_D T plm_limit(T s, T l, T r) {
  if (l * r > T(0)) {
    const T m = fmin(fabs(s), fmin(T(2) * fabs(l), T(2) * fabs(r)));
    return s >= T(0) ? m : -m;
  }
  return T(0);
}

// PLM normal predictor of one side of one cell (characteristic tracing
// dWm = -1/2 (1 + min(sig, 0)) dW, dWp = 1/2 (1 - max(sig, 0)) dW, Colella 1990)
template <int D, typename T>
TMK_D void plm_predict(const Consts<T>& k, T rv, const T (*w5)[5], const bool* in, bool prim_lim, bool char_lim,
                       bool fourth, const T* sig, T* WM, T* WP) {
  const bool limit = prim_lim || char_lim;
  T dW[NSIDE], dm[NSIDE], dp[NSIDE];
#pragma unroll
  for (int c = 0; c < NSIDE; ++c) {
    dW[c] = plm_slope(w5[c], in, limit, fourth);
    dm[c] = T(0); dp[c] = T(0);
    if (char_lim || fourth) plm_onesided(w5[c], in, dm[c], dp[c]);
  }
  T cW[NSIDE];
  if (char_lim) {
    T cm[NSIDE], cp[NSIDE];
    char_analysis<D>(k, rv, dm, cm);
    char_analysis<D>(k, rv, dp, cp);
    char_analysis<D>(k, rv, dW, cW);
#pragma unroll
    for (int c = 0; c < NSIDE; ++c) cW[c] = plm_limit(cW[c], cm[c], cp[c]);
  } else {
    if (prim_lim && fourth) {
#pragma unroll
      for (int c = 0; c < NSIDE; ++c) dW[c] = plm_limit(dW[c], dm[c], dp[c]);
    }
    char_analysis<D>(k, rv, dW, cW);
  }
  T cmo[NSIDE], cpo[NSIDE];
#pragma unroll
  for (int c = 0; c < NSIDE; ++c) {
    cmo[c] = -T(0.5) * (T(1) + fmin(sig[c], T(0))) * cW[c];
    cpo[c] = T(0.5) * (T(1) - fmax(sig[c], T(0))) * cW[c];
  }
  char_synthesis<D>(k, rv, cmo, WM);
  char_synthesis<D>(k, rv, cpo, WP);
#pragma unroll
  for (int c = 0; c < NSIDE; ++c) { WM[c] += w5[c][2]; WP[c] += w5[c][2]; }
}

// Normal predictor of one side of one cell in direction D (order 2: PPM;
// order 1: PLM; order 0: CTUNormalPred, a straight copy of the cell state to
// both faces, srcLinElast/LinElastPatchGodunov.cpp:471-483).
// Full PPM normal predictor of one side of one cell in direction D:
// w5[c][k] holds component c at cells -2..+2.  Produces WM (lo face) and WP.
// sig[9] are the characteristic Courant numbers (-cp,-cs,-cs,0,0,0,cs,cs,cp)*dt/dx.
template <int D, typename T>
TMK_D void ppm_predict(const Consts<T>& k, T rv, const T (*w5)[5], const bool* in, bool prim_lim,
                       bool char_lim, const T* sig, T* WM, T* WP, int order = 2, bool fourth = false) {
  if (order == 0) {
#pragma unroll
    for (int c = 0; c < NSIDE; ++c) { WM[c] = w5[c][2]; WP[c] = w5[c][2]; }
    return;
  }
  if (order == 1) {
    plm_predict<D, T>(k, rv, w5, in, prim_lim, char_lim, fourth, sig, WM, WP);
    return;
  }
  T dm[NSIDE], dp[NSIDE];
  const bool limit = prim_lim || char_lim;
#pragma unroll
  for (int c = 0; c < NSIDE; ++c) ppm_deltas(w5[c], in, limit, dm[c], dp[c]);
  T cm[NSIDE], cpv[NSIDE];
  if (char_lim) {
    char_analysis<D>(k, rv, dm, cm);
    char_analysis<D>(k, rv, dp, cpv);
#pragma unroll
    for (int c = 0; c < NSIDE; ++c) ppm_limit(cm[c], cpv[c]);
  } else {
    if (prim_lim) {
#pragma unroll
      for (int c = 0; c < NSIDE; ++c) ppm_limit(dm[c], dp[c]);
    }
    char_analysis<D>(k, rv, dm, cm);
    char_analysis<D>(k, rv, dp, cpv);
  }
#pragma unroll
  for (int c = 0; c < NSIDE; ++c) ppm_trace(sig[c], cm[c], cpv[c]);
  char_synthesis<D>(k, rv, cm, WM);
  char_synthesis<D>(k, rv, cpv, WP);
#pragma unroll
  for (int c = 0; c < NSIDE; ++c) { WM[c] += w5[c][2]; WP[c] += w5[c][2]; }
}

// PPM normal predictor of one side of one cell with primitive limiting, for
// the mixed forms (the 3-D passes, the fault-row predictors): the stages of ppm_predict with the domain-edge cases as
// selects instead of branches (a warp along x holds edge and inner cells), and
// the tracing of each characteristic with the coefficients of its known
// direction -- the waves (-cp, -cs, -cs) move to the lo face, (cs, cs, cp) to
// the hi face:
//   lo-going  m <- m + A (p - m) - B (m + p),  A = s/2, B = 3 (s/2 - s^2/3)
//   hi-going  p <- p - A (p - m) - B (m + p),  A = s/2, B = (3/2) s (1 - 2s/3)
// with s = |lambda| dt/dx (Colella & Woodward 1984 eq. 1.12).
// Van Leer limited slope of w0 with neighbours wm, wp (one-sided next to a
// domain edge, zero with neither neighbour)
template <typename T>
TMK_D T vl_lim(T wm, T w0, T wp, bool hasL, bool hasR) {
  const T dL = w0 - wm, dR = wp - w0;
  const T dl = hasL ? dL : dR, dr = hasR ? dR : dL;
  const T dc = (hasL && hasR) ? T(0.5) * (wp - wm) : dl;
  const T m = fmin(fabs(dc), T(2) * fmin(fabs(dl), fabs(dr)));
  return (dl * dr > T(0) && (hasL || hasR)) ? copysign(m, dc) : T(0);
}

// the characteristic stage of ppm_predict_prim: limited deltas dm, dp of the
// cell with centre values w -> traced face states WM, WP
template <int D, typename T>
TMK_D void prim_trace(const Consts<T>& k, T rv, const T* dm, const T* dp, const T* w, const T* trA, const T* trB,
                      T* WM, T* WP) {
  T cm[NSIDE], cp[NSIDE];
  char_analysis<D>(k, rv, dm, cm);
  char_analysis<D>(k, rv, dp, cp);
#pragma unroll
  for (int c = 0; c < 3; ++c) cm[c] = cm[c] + trA[c] * (cp[c] - cm[c]) - trB[c] * (cm[c] + cp[c]);
#pragma unroll
  for (int c = 6; c < 9; ++c) cp[c] = cp[c] - trA[c] * (cp[c] - cm[c]) - trB[c] * (cm[c] + cp[c]);
  char_synthesis<D>(k, rv, cm, WM);
  char_synthesis<D>(k, rv, cp, WP);
#pragma unroll
  for (int c = 0; c < NSIDE; ++c) { WM[c] += w[c]; WP[c] += w[c]; }
}

template <int D, typename T>
TMK_D void ppm_predict_prim(const Consts<T>& k, T rv, const T (*w5)[5], const bool* in, const T* trA, const T* trB,
                            T* WM, T* WP) {
  T dm[NSIDE], dp[NSIDE], w[NSIDE];
#pragma unroll
  for (int c = 0; c < NSIDE; ++c) {
    const T* wc = w5[c];
    const T sm = in[1] ? vl_lim(wc[0], wc[1], wc[2], in[0], true) : T(0);
    const T s0 = vl_lim(wc[1], wc[2], wc[3], in[1], in[3]);
    const T sp = in[3] ? vl_lim(wc[2], wc[3], wc[4], true, in[4]) : T(0);
    const T flo = in[1] ? T(0.5) * (wc[1] + wc[2]) - (s0 - sm) * T(1.0 / 6.0) : wc[2] - T(0.5) * s0;
    const T fhi = in[3] ? T(0.5) * (wc[2] + wc[3]) - (sp - s0) * T(1.0 / 6.0) : wc[2] + T(0.5) * s0;
    T m = flo - wc[2], p = fhi - wc[2];
    ppm_limit(m, p);
    dm[c] = m; dp[c] = p; w[c] = wc[2];
  }
  prim_trace<D, T>(k, rv, dm, dp, w, trA, trB, WM, WP);
}

// ppm_predict_prim for two neighbouring cells along D (window points 2 and 3 of
// w6, in[m] whether point m lies in the domain; the second cell only if `two`,
// which implies in[3]): the slopes at points 2 and 3 and the face value
// between the cells serve both, with the same arithmetic as two single calls.
template <int D, typename T>
TMK_D void ppm_predict_prim2(const Consts<T>& k, T rv, const T (*w6)[6], const bool* in, bool two, const T* trA,
                             const T* trB, T* WM0, T* WP0, T* WM1, T* WP1) {
  T dm0[NSIDE], dp0[NSIDE], dm1[NSIDE], dp1[NSIDE], w0[NSIDE], w1[NSIDE];
#pragma unroll
  for (int c = 0; c < NSIDE; ++c) {
    const T* w = w6[c];
    const T s1 = in[1] ? vl_lim(w[0], w[1], w[2], in[0], true) : T(0);
    const T s2 = vl_lim(w[1], w[2], w[3], in[1], in[3]);
    const T s3 = in[3] ? vl_lim(w[2], w[3], w[4], true, in[4]) : T(0);
    const T f12 = in[1] ? T(0.5) * (w[1] + w[2]) - (s2 - s1) * T(1.0 / 6.0) : w[2] - T(0.5) * s2;
    const T f23 = in[3] ? T(0.5) * (w[2] + w[3]) - (s3 - s2) * T(1.0 / 6.0) : w[2] + T(0.5) * s2;
    T m = f12 - w[2], p = f23 - w[2];
    ppm_limit(m, p);
    dm0[c] = m; dp0[c] = p; w0[c] = w[2];
    const T s4 = in[4] ? vl_lim(w[3], w[4], w[5], true, in[5]) : T(0);
    const T f34 = in[4] ? T(0.5) * (w[3] + w[4]) - (s4 - s3) * T(1.0 / 6.0) : w[3] + T(0.5) * s3;
    T m1 = f23 - w[3], p1 = f34 - w[3];
    ppm_limit(m1, p1);
    dm1[c] = m1; dp1[c] = p1; w1[c] = w[3];
  }
  prim_trace<D, T>(k, rv, dm0, dp0, w0, trA, trB, WM0, WP0);
  if (two) prim_trace<D, T>(k, rv, dm1, dp1, w1, trA, trB, WM1, WP1);
}

// -------------------------------------------------------- status reporting
enum : int { ST_OK = 0, ST_NAN = 2, ST_TIMEOUT = 3 };
struct DevStatus {
  int code;                 // first error code (0 = none)
  int pad;
  long long first_index;    // flat index of the first bad value
  unsigned long long newton_maxed;   // Newton solves that used all IMAX iterations
};

TMK_D void report(DevStatus* st, int code, long long idx) {
  if (atomicCAS(&st->code, 0, code) == 0) st->first_index = idx;
}

}  // namespace tmk
