// The 3-D patch step (CH_SPACEDIM == 3), FP64.  Compiled with --fmad=false
// so that every product and sum rounds as in the reference's Fortran and the
// CPU oracle.
//
// LinElastPatchGodunov::updateState in 3-D (srcLinElast/LinElastPatchGodunov.cpp:
// 101-129, 174-469) as five kinds of passes over one patch, each a grid of one
// thread per cell or face, with the intermediates in device scratch:
//   pred<D>      normal predictor in direction D on the slope box (both sides
//                of the fault packed as 18 components: the nine evolving
//                components of each side; lambda and gamma carry no flux)
//   riem1<D>     first-pass face states WHalf1[D] (Riemann solve, or the
//                domain-edge / fault condition)
//   riem2<D1,D2> WHalf2[D1][D2]: the D1 face states after the normal states
//                were moved by -(1/3) dt/dx A dW/dx of WHalf1[D2] (:329-381)
//   final<D1>    the time-centred WHalf[D1], normal states moved by both
//                WHalf2[D2][D3] with -(1/2) dt/dx (:422-440)
//   update       fluxes, their divergence and U += -dt/dx dU in place; then
//                the fault's boundary data (RSSETBND / SWSETBND, final)
// The fault is the y-lo plane of the domain.  Its boundary data predicted at
// (1/3) dt from WHalf1[1] and at (1/2) dt from WHalf2[1][2] (the reference's
// call order leaves those in m_tmpBdryData when WHalf2[1][*] and WHalf[1] are
// solved) are formed at the face that reads them.  Fault faces keep all 22
// components of their states beside the 18-component arrays, because the
// reference-layout slip-weakening law reads and writes side 2 from component 9.
#include <algorithm>
#include <cstring>
#include <vector>

#include "tmk_internal.h"
#include "tmk_kernels.cuh"

namespace tmk {
namespace d3 {

constexpr int NS = 2 * NSIDE;     // 18 stored components

struct Bx {
  int lo[3], n[3];
  TMK_HD long long cells() const { return (long long)n[0] * n[1] * n[2]; }
  TMK_HD bool has(int i, int j, int k) const {
    return i >= lo[0] && i < lo[0] + n[0] && j >= lo[1] && j < lo[1] + n[1] && k >= lo[2] && k < lo[2] + n[2];
  }
  TMK_HD long long at(int i, int j, int k) const {
    return ((long long)(k - lo[2]) * n[1] + (j - lo[1])) * n[0] + (i - lo[0]);
  }
  TMK_HD void cell(long long t, int& i, int& j, int& k) const {
    i = lo[0] + (int)(t % n[0]);
    long long r = t / n[0];
    j = lo[1] + (int)(r % n[1]);
    k = lo[2] + (int)(r / n[1]);
  }
};

struct Step3 {
  Bx A;                 // U's box
  Bx S;                 // slope box: grow(valid, 1) & domain
  Bx fl1[3];            // first-pass faces: nodes(ccBox[d], d)
  Bx cc[3];             // ccBox[d]: grow(valid, 1) shrunk by 1 in d, & domain
  Bx flF[3];            // final faces: nodes(valid, d)
  Bx cur;
  int dlo[3], dhi[3];
  Bx fplane;            // fault faces of the first pass (x, z of fl1[1]; j = domain lo)
  Bx bb;                // B's box (j = domain lo)
  double* U;
  double* WM[3];
  double* WP[3];
  double* WH1[3];
  double* WH2[3][3];    // WHalf2[d1][d2], d1 != d2
  double* WH[3];
  double* LG;           // lambda, gamma of side 1 predicted at the fault's lo faces (fplane)
  double* FF[3];        // 22-comp fault-face states of WHalf1[1], WHalf2[1][2], WHalf[1] (fplane)
  double* B;
  double* F[3];         // optional face fluxes (22 comps over flF[d])
  double dx, dt, time;
  int fault;
};

template <int D> TMK_HD double rvs(int s) { return (D == 1 && s == 1) ? -1.0 : 1.0; }

TMK_D void load18(const double* a, const Bx& b, int i, int j, int k, double* q) {
  const long long cs = b.cells(), o = b.at(i, j, k);
#pragma unroll
  for (int c = 0; c < NS; ++c) q[c] = a[c * cs + o];
}
TMK_D void store18(double* a, const Bx& b, int i, int j, int k, const double* q) {
  const long long cs = b.cells(), o = b.at(i, j, k);
#pragma unroll
  for (int c = 0; c < NS; ++c) a[c * cs + o] = q[c];
}
template <int D> TMK_D void step(int& i, int& j, int& k, int s) {
  if (D == 0) i += s; else if (D == 1) j += s; else k += s;
}
template <int D> TMK_D int coord(int i, int j, int k) { return D == 0 ? i : (D == 1 ? j : k); }

// Predicted lo-face value of a zero-speed component (lambda or gamma) in the
// arithmetic of ppm_predict / plm_predict: PPM limited delta, PLM traced slope,
// or the cell value (CTU).
TMK_D double zero_speed_lo(const DevParams& P, const double* w, const bool* in) {
  const bool lim = P.prim_lim || P.char_lim;
  if (P.order == 0) return w[2];
  if (P.order == 1) {
    double sl = plm_slope(w, in, lim, P.fourth != 0);
    if (lim && (P.char_lim || P.fourth)) {
      double m, p1;
      plm_onesided(w, in, m, p1);
      sl = plm_limit(sl, m, p1);
    }
    return -0.5 * sl + w[2];
  }
  double dm, dp;
  ppm_deltas(w, in, lim, dm, dp);
  if (lim) ppm_limit(dm, dp);
  return dm + w[2];
}

// ------------------------------------------------------------- predictors
template <int D>
__global__ void __launch_bounds__(128) pred_kernel(const __grid_constant__ Step3 g, const DevParams* Pp) {
  const DevParams& P = *Pp;
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= g.S.cells()) return;
  int i, j, k;
  g.S.cell(t, i, j, k);
  Consts<double> kc;
  kc.load(P);
  double sig[NSIDE];
  make_sig(P, g.dt / g.dx, sig);
  const int q0 = coord<D>(i, j, k);
  bool in[5];
#pragma unroll
  for (int m = 0; m < 5; ++m) in[m] = q0 - 2 + m >= g.dlo[D] && q0 - 2 + m <= g.dhi[D];
  const long long acs = g.A.cells();
  double WM[NS], WP[NS];
#pragma unroll
  for (int s = 0; s < 2; ++s) {
    double w5[NSIDE][5];
#pragma unroll
    for (int m = 0; m < 5; ++m) {
      int ii = i, jj = j, kk = k;
      step<D>(ii, jj, kk, m - 2);
      const long long o = in[m] ? g.A.at(ii, jj, kk) : 0;
#pragma unroll
      for (int c = 0; c < NSIDE; ++c) w5[c][m] = in[m] ? g.U[(11 * s + c) * acs + o] : 0.0;
    }
    ppm_predict<D, double>(kc, rvs<D>(s), w5, in, P.prim_lim != 0, P.char_lim != 0, sig, WM + NSIDE * s,
                           WP + NSIDE * s, P.order, P.fourth != 0);
  }
  store18(g.WM[D], g.S, i, j, k, WM);
  store18(g.WP[D], g.S, i, j, k, WP);
  if (D == 1 && g.fault && j == g.dlo[1]) {
    // lambda and gamma of side 1 at the fault's lo faces (read by the
    // reference-layout slip-weakening law as side-2 velocities)
#pragma unroll
    for (int c = 9; c < 11; ++c) {
      double w[5];
#pragma unroll
      for (int m = 0; m < 5; ++m) {
        int ii = i, jj = j, kk = k;
        step<D>(ii, jj, kk, m - 2);
        w[m] = in[m] ? g.U[c * acs + g.A.at(ii, jj, kk)] : 0.0;
      }
      g.LG[(c - 9) * g.fplane.cells() + g.fplane.at(i, j, k)] = zero_speed_lo(P, w, in);
    }
  }
}

// -------------------------------------------------------- face conditions
// Boundary data value the fault law reads at face (i, k): psi (rate and
// state) or slip (slip weakening), from B, or from B moved by the 22-comp face
// state U22 over `dtp` (the predictor's m_tmpBdryData, updateBoundary final=false).
TMK_D double bdry_value(const DevParams& P, const Step3& g, int i, int k, const double* U22, double dtp) {
  double* Bi = g.B + g.bb.at(i, g.dlo[1], k);
  const long long bs = g.bb.cells();
  if (!U22) return P.fault_law == 1 ? Bi[10 * bs] : Bi[7 * bs];
  if (P.fault_law == 1) {
    const RSFace fr = rs_face(P, nullptr, 0, 0);
    return rs_setbnd(P, fr, U22, Bi, (int)bs, dtp, (i + 0.5) * g.dx - P.rs_x0, 0.0, false);
  }
  return sw_setbnd(P, U22, Bi, (int)bs, dtp, 0.0, false);
}

// fault face (i, dom lo, k): 22-comp state Wg from the interior state Wi22
TMK_D void fault_face(const DevParams& P, const Step3& g, int i, int k, const double* Wi, double bval, double* Wg,
                      DevStatus* st) {
#pragma unroll
  for (int c = 0; c < NC; ++c) Wg[c] = 0.0;
  const double xc = (i + 0.5) * g.dx;
  if (P.fault_law == 1) {
    const RSFace fr = rs_face(P, nullptr, 0, 0);
    const int it = rs_fault(P, fr, Wi, bval, xc - P.rs_x0, Wg);
    if (it > RS_IMAX) atomicAdd(&st->newton_maxed, 1ull);
  } else {
    sw_fault<true>(P, Wi, bval, xc, Wg, (k + 0.5) * g.dx);
  }
}

// Face f of direction D with left cell state L18 and right cell state R18:
// Riemann solve, or the domain-edge condition.  Returns false for the fault
// faces (y lo with a fault law), which the caller solves.
template <int D>
TMK_D bool face_state(const DevParams& P, const Consts<double>& kc, const Step3& g, int f, const double* L18,
                      const double* R18, double* G18) {
  if (f == g.dlo[D]) {
    if (D == 1 && g.fault) return false;
    const bool outflow = P.bc[2 * D] == 0;
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      double bg[NSIDE];
      side_bg(P, s, bg);
      edge_bc<D, double>(kc, rvs<D>(s), -1, outflow, bg, R18 + NSIDE * s, G18 + NSIDE * s);
    }
  } else if (f == g.dhi[D] + 1) {
    const bool outflow = P.bc[2 * D + 1] == 0;
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      double bg[NSIDE];
      side_bg(P, s, bg);
      edge_bc<D, double>(kc, rvs<D>(s), +1, outflow, bg, L18 + NSIDE * s, G18 + NSIDE * s);
    }
  } else {
#pragma unroll
    for (int s = 0; s < 2; ++s) riemann<D, double>(kc, rvs<D>(s), L18 + NSIDE * s, R18 + NSIDE * s, G18 + NSIDE * s);
  }
  return true;
}

// fault face: gather the 22-comp interior state, solve, keep 22 comps in FFk
TMK_D void fault_solve(const DevParams& P, const Step3& g, int i, int k, const double* R18, double bval,
                       double* FFk, double* G18, DevStatus* st) {
  double Wi[NC], Wg[NC];
  const long long fo = g.fplane.at(i, g.dlo[1], k), fcs = g.fplane.cells();
#pragma unroll
  for (int c = 0; c < NSIDE; ++c) { Wi[c] = R18[c]; Wi[11 + c] = R18[NSIDE + c]; }
  Wi[9] = g.LG[fo]; Wi[10] = g.LG[fcs + fo];
  Wi[20] = 0.0; Wi[21] = 0.0;
  fault_face(P, g, i, k, Wi, bval, Wg, st);
#pragma unroll
  for (int c = 0; c < NSIDE; ++c) { G18[c] = Wg[c]; G18[NSIDE + c] = Wg[11 + c]; }
  if (FFk) {
#pragma unroll
    for (int c = 0; c < NC; ++c) FFk[c * fcs + fo] = Wg[c];
  }
}

TMK_D void load_ff(const Step3& g, const double* FFk, int i, int k, double* U22) {
  const long long fo = g.fplane.at(i, g.dlo[1], k), fcs = g.fplane.cells();
#pragma unroll
  for (int c = 0; c < NC; ++c) U22[c] = FFk[c * fcs + fo];
}

// ------------------------------------------------------------ first pass
template <int D>
__global__ void __launch_bounds__(128) riem1_kernel(const __grid_constant__ Step3 g, const DevParams* Pp,
                                                    DevStatus* st) {
  const DevParams& P = *Pp;
  const Bx& fb = g.fl1[D];
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= fb.cells()) return;
  int i, j, k;
  fb.cell(t, i, j, k);
  Consts<double> kc;
  kc.load(P);
  const int f = coord<D>(i, j, k);
  double L[NS], R[NS], G[NS];
  int li = i, lj = j, lk = k;
  step<D>(li, lj, lk, -1);
  if (f > g.dlo[D]) load18(g.WP[D], g.S, li, lj, lk, L);
  if (f <= g.dhi[D]) load18(g.WM[D], g.S, i, j, k, R);
  if (!face_state<D>(P, kc, g, f, L, R, G))
    fault_solve(P, g, i, k, R, bdry_value(P, g, i, k, nullptr, 0.0), g.FF[0], G, st);
  store18(g.WH1[D], fb, i, j, k, G);
}

// cell state T18 of array A (direction-D1 normal states) at (i, j, k), moved by
// -(scale) A dW/dx of the face states H in direction D2 where the cell lies in ccBox[D2]
template <int D2>
TMK_D void corrected(const Step3& g, const Consts<double>& kc, const double* A, const double* H, const Bx& hb,
                     double scale, int i, int j, int k, double* T18) {
  load18(A, g.S, i, j, k, T18);
  if (!g.cc[D2].has(i, j, k)) return;
  double h[NS], l[NS];
  int hi = i, hj = j, hk = k;
  step<D2>(hi, hj, hk, 1);
  load18(H, hb, hi, hj, hk, h);
  load18(H, hb, i, j, k, l);
#pragma unroll
  for (int s = 0; s < 2; ++s) adwdx_add<D2, double>(kc, rvs<D2>(s), scale, h + NSIDE * s, l + NSIDE * s, T18 + NSIDE * s);
}

// ----------------------------------------------------------- second pass
template <int D1, int D2>
__global__ void __launch_bounds__(128) riem2_kernel(const __grid_constant__ Step3 g, const DevParams* Pp,
                                                    DevStatus* st) {
  const DevParams& P = *Pp;
  const Bx& fb = g.fl1[D1];
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= fb.cells()) return;
  int i, j, k;
  fb.cell(t, i, j, k);
  Consts<double> kc;
  kc.load(P);
  const double scale = -(1.0 / 3.0) * g.dt / g.dx;
  const int f = coord<D1>(i, j, k);
  double L[NS], R[NS], G[NS];
  int li = i, lj = j, lk = k;
  step<D1>(li, lj, lk, -1);
  if (f > g.dlo[D1]) corrected<D2>(g, kc, g.WP[D1], g.WH1[D2], g.fl1[D2], scale, li, lj, lk, L);
  if (f <= g.dhi[D1]) corrected<D2>(g, kc, g.WM[D1], g.WH1[D2], g.fl1[D2], scale, i, j, k, R);
  if (!face_state<D1>(P, kc, g, f, L, R, G)) {
    double U22[NC];
    load_ff(g, g.FF[0], i, k, U22);
    const double bval = bdry_value(P, g, i, k, U22, (1.0 / 3.0) * g.dt);
    fault_solve(P, g, i, k, R, bval, (D2 == 2) ? g.FF[1] : nullptr, G, st);
  }
  store18(g.WH2[D1][D2], fb, i, j, k, G);
}

// ------------------------------------------------------------ final pass
template <int D1>
TMK_D void final_state(const Step3& g, const Consts<double>& kc, const double* A, double scale, int i, int j, int k,
                       double* T18) {
  constexpr int Da = (D1 == 0) ? 1 : 0;      // the two other directions, ascending
  constexpr int Db = (D1 == 2) ? 1 : 2;
  load18(A, g.S, i, j, k, T18);
  double h[NS], l[NS];
  if (g.cc[Da].has(i, j, k)) {
    constexpr int D3 = 3 - D1 - Da;
    int hi = i, hj = j, hk = k;
    step<Da>(hi, hj, hk, 1);
    load18(g.WH2[Da][D3], g.fl1[Da], hi, hj, hk, h);
    load18(g.WH2[Da][D3], g.fl1[Da], i, j, k, l);
#pragma unroll
    for (int s = 0; s < 2; ++s) adwdx_add<Da, double>(kc, rvs<Da>(s), scale, h + NSIDE * s, l + NSIDE * s, T18 + NSIDE * s);
  }
  if (g.cc[Db].has(i, j, k)) {
    constexpr int D3 = 3 - D1 - Db;
    int hi = i, hj = j, hk = k;
    step<Db>(hi, hj, hk, 1);
    load18(g.WH2[Db][D3], g.fl1[Db], hi, hj, hk, h);
    load18(g.WH2[Db][D3], g.fl1[Db], i, j, k, l);
#pragma unroll
    for (int s = 0; s < 2; ++s) adwdx_add<Db, double>(kc, rvs<Db>(s), scale, h + NSIDE * s, l + NSIDE * s, T18 + NSIDE * s);
  }
}

template <int D1>
__global__ void __launch_bounds__(128) final_kernel(const __grid_constant__ Step3 g, const DevParams* Pp,
                                                    DevStatus* st) {
  const DevParams& P = *Pp;
  const Bx& fb = g.flF[D1];
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= fb.cells()) return;
  int i, j, k;
  fb.cell(t, i, j, k);
  Consts<double> kc;
  kc.load(P);
  const double scale = -(1.0 / 2.0) * g.dt / g.dx;
  const int f = coord<D1>(i, j, k);
  double L[NS], R[NS], G[NS];
  int li = i, lj = j, lk = k;
  step<D1>(li, lj, lk, -1);
  if (f > g.dlo[D1]) final_state<D1>(g, kc, g.WP[D1], scale, li, lj, lk, L);
  if (f <= g.dhi[D1]) final_state<D1>(g, kc, g.WM[D1], scale, i, j, k, R);
  if (!face_state<D1>(P, kc, g, f, L, R, G)) {
    double U22[NC];
    load_ff(g, g.FF[1], i, k, U22);
    const double bval = bdry_value(P, g, i, k, U22, (1.0 / 2.0) * g.dt);
    fault_solve(P, g, i, k, R, bval, g.FF[2], G, st);
  }
  store18(g.WH[D1], fb, i, j, k, G);
}

// ---------------------------------------------------------------- update
template <int D>
TMK_D void flux_diff(const Step3& g, const Consts<double>& kc, int i, int j, int k, double* dU) {
  double h[NS], l[NS], Fh[NS], Fl[NS];
  int hi = i, hj = j, hk = k;
  step<D>(hi, hj, hk, 1);
  load18(g.WH[D], g.flF[D], hi, hj, hk, h);
  load18(g.WH[D], g.flF[D], i, j, k, l);
#pragma unroll
  for (int s = 0; s < 2; ++s) {
    flux<D, double>(kc, rvs<D>(s), h + NSIDE * s, Fh + NSIDE * s);
    flux<D, double>(kc, rvs<D>(s), l + NSIDE * s, Fl + NSIDE * s);
  }
#pragma unroll
  for (int c = 0; c < NS; ++c) dU[c] += Fh[c] - Fl[c];
}

__global__ void __launch_bounds__(128) update_kernel(const __grid_constant__ Step3 g, const DevParams* Pp) {
  const DevParams& P = *Pp;
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= g.cur.cells()) return;
  int i, j, k;
  g.cur.cell(t, i, j, k);
  Consts<double> kc;
  kc.load(P);
  double dU[NS];
#pragma unroll
  for (int c = 0; c < NS; ++c) dU[c] = 0.0;
  flux_diff<0>(g, kc, i, j, k, dU);
  flux_diff<1>(g, kc, i, j, k, dU);
  flux_diff<2>(g, kc, i, j, k, dU);
  const double sc = -g.dt / g.dx;
  const long long acs = g.A.cells(), o = g.A.at(i, j, k);
#pragma unroll
  for (int s = 0; s < 2; ++s)
#pragma unroll
    for (int c = 0; c < NSIDE; ++c) {
      double* u = g.U + (11 * s + c) * acs + o;
      *u = *u + dU[NSIDE * s + c] * sc;
    }
}

// the face fluxes of direction D (22 comps; lambda, gamma and the antiplane
// stress of the face normal carry none)
template <int D>
__global__ void __launch_bounds__(128) flux_kernel(const __grid_constant__ Step3 g, const DevParams* Pp) {
  const DevParams& P = *Pp;
  const Bx& fb = g.flF[D];
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= fb.cells()) return;
  int i, j, k;
  fb.cell(t, i, j, k);
  Consts<double> kc;
  kc.load(P);
  double w[NS], F[NS];
  load18(g.WH[D], fb, i, j, k, w);
#pragma unroll
  for (int s = 0; s < 2; ++s) flux<D, double>(kc, rvs<D>(s), w + NSIDE * s, F + NSIDE * s);
  const long long cs = fb.cells();
  double* out = g.F[D] + t;
#pragma unroll
  for (int s = 0; s < 2; ++s) {
#pragma unroll
    for (int c = 0; c < NSIDE; ++c) out[(11 * s + c) * cs] = F[NSIDE * s + c];
    out[(11 * s + 9) * cs] = 0.0;
    out[(11 * s + 10) * cs] = 0.0;
  }
}

// the fault's boundary data, final (RSSETBND / SWSETBND over the valid x, z)
__global__ void __launch_bounds__(128) bdry_final_kernel(const __grid_constant__ Step3 g, const DevParams* Pp,
                                                         DevStatus* st) {
  const DevParams& P = *Pp;
  const int nx = g.cur.n[0], nz = g.cur.n[2];
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= (long long)nx * nz) return;
  const int i = g.cur.lo[0] + (int)(t % nx), k = g.cur.lo[2] + (int)(t / nx);
  double U22[NC];
  load_ff(g, g.FF[2], i, k, U22);
  const long long bo = g.bb.at(i, g.dlo[1], k);
  double* Bi = g.B + bo;
  const int bs = (int)g.bb.cells();
  if (P.fault_law == 1) {
    const RSFace fr = rs_face(P, nullptr, 0, 0);
    const double psi = rs_setbnd(P, fr, U22, Bi, bs, g.dt, (i + 0.5) * g.dx - P.rs_x0, g.time + g.dt, true);
    if (isnan(psi)) report(st, ST_NAN, bo);
  } else {
    sw_setbnd(P, U22, Bi, bs, g.dt, g.time + g.dt, true);
  }
}

__global__ void plastic3_kernel(double* U, Bx A, Bx box, const DevParams* P, double dt) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= box.cells()) return;
  int i, j, k;
  box.cell(t, i, j, k);
  const long long cs = A.cells(), o = A.at(i, j, k);
  for (int s = 0; s < 2; ++s) {
    double* u = U + (11 * s) * cs + o;
    double sxx = u[3 * cs], syy = u[4 * cs], szz = u[5 * cs], sxy = u[6 * cs];
    double sxz = u[7 * cs], syz = u[8 * cs], lam = u[9 * cs], gam = u[10 * cs];
    plastic_flow<double>(*P, sxx, syy, szz, sxy, sxz, syz, lam, gam, dt);
    u[3 * cs] = sxx; u[4 * cs] = syy; u[5 * cs] = szz; u[6 * cs] = sxy;
    u[7 * cs] = sxz; u[8 * cs] = syz; u[9 * cs] = lam; u[10 * cs] = gam;
  }
}

inline unsigned blocks(long long n) { return (unsigned)((n + 127) / 128); }

}  // namespace d3
}  // namespace tmk

// ==================================================================== C ABI
namespace {

using tmk::d3::Bx;

Bx bx_of(const int lo[3], const int hi[3]) {
  Bx b;
  for (int d = 0; d < 3; ++d) { b.lo[d] = lo[d]; b.n[d] = hi[d] - lo[d] + 1; }
  return b;
}
bool bx_ok(const Bx& b) { return b.n[0] > 0 && b.n[1] > 0 && b.n[2] > 0; }
int bx_hi(const Bx& b, int d) { return b.lo[d] + b.n[d] - 1; }
bool bx_contains(const Bx& a, const Bx& b) {
  for (int d = 0; d < 3; ++d)
    if (b.lo[d] < a.lo[d] || bx_hi(b, d) > bx_hi(a, d)) return false;
  return true;
}
Bx bx_grow(Bx b, int d, int n) { b.lo[d] -= n; b.n[d] += 2 * n; return b; }
Bx bx_grow(Bx b, int n) { for (int d = 0; d < 3; ++d) b = bx_grow(b, d, n); return b; }
Bx bx_isect(Bx a, const Bx& b) {
  for (int d = 0; d < 3; ++d) {
    int lo = std::max(a.lo[d], b.lo[d]), hi = std::min(bx_hi(a, d), bx_hi(b, d));
    a.lo[d] = lo; a.n[d] = hi - lo + 1;
  }
  return a;
}
Bx bx_nodes(Bx b, int d) { b.n[d] += 1; return b; }

size_t align_up3(size_t v) { return (v + 255) & ~(size_t)255; }

}  // namespace

extern "C" tmk_status tmk_patch_update_state_3d(tmk_context* c, const tmk_fab3* U, const tmk_fab3* B,
                                                const tmk_fab3* F0, const tmk_fab3* F1, const tmk_fab3* F2,
                                                const tmk_box3* valid, const tmk_box3* domain, double dx,
                                                double time, double dt, double* max_wave_speed, void* stream) {
  using namespace tmk::d3;
  if (!c || !U || !U->data || !valid || !domain) return TMK_ERR_BAD_DESC;
  if (U->ncomp != TMK_NCOMP || !(dx > 0) || !(dt > 0)) return TMK_ERR_BAD_DESC;
  const Bx cur = bx_of(valid->lo, valid->hi), dom = bx_of(domain->lo, domain->hi), A = bx_of(U->lo, U->hi);
  if (!bx_ok(cur) || !bx_ok(dom) || !bx_ok(A) || !bx_contains(dom, cur)) return TMK_ERR_BAD_DESC;
  if (!bx_contains(A, bx_isect(bx_grow(cur, 3), dom))) return TMK_ERR_BAD_DESC;
  Step3 g;
  std::memset(&g, 0, sizeof(g));
  g.A = A; g.cur = cur;
  for (int d = 0; d < 3; ++d) { g.dlo[d] = domain->lo[d]; g.dhi[d] = domain->hi[d]; }
  g.S = bx_isect(bx_grow(cur, 1), dom);
  for (int d = 0; d < 3; ++d) {
    g.cc[d] = bx_isect(bx_grow(bx_grow(cur, 1), d, -1), dom);
    g.fl1[d] = bx_nodes(g.cc[d], d);
    g.flF[d] = bx_nodes(cur, d);
  }
  g.fault = c->scheme.fault_law != TMK_FAULT_NONE && cur.lo[1] == dom.lo[1];
  g.fplane = g.fl1[1];
  g.fplane.n[1] = 1;
  if (g.fault) {
    if (!B || !B->data || B->ncomp != c->nb || B->lo[1] != dom.lo[1] || B->hi[1] != dom.lo[1]) return TMK_ERR_BAD_DESC;
    g.bb = bx_of(B->lo, B->hi);
    if (!bx_contains(g.bb, g.fplane)) return TMK_ERR_BAD_DESC;
    g.B = B->data;
  }
  const tmk_fab3* Fo[3] = {F0, F1, F2};
  for (int d = 0; d < 3; ++d) {
    if (!Fo[d]) continue;
    if (!Fo[d]->data || Fo[d]->ncomp != TMK_NCOMP) return TMK_ERR_BAD_DESC;
    const Bx fb = bx_of(Fo[d]->lo, Fo[d]->hi);
    for (int e = 0; e < 3; ++e)
      if (fb.lo[e] != g.flF[d].lo[e] || fb.n[e] != g.flF[d].n[e]) return TMK_ERR_BAD_DESC;
    g.F[d] = Fo[d]->data;
  }
  g.U = U->data;
  g.dx = dx; g.dt = dt; g.time = time;

  // scratch: WM, WP (3 each) | WH1 (3) | WH2 (6) | WH (3) | LG | FF (3)
  const size_t s18 = (size_t)NS * g.S.cells() * sizeof(double);
  std::vector<size_t> sizes;
  for (int d = 0; d < 6; ++d) sizes.push_back(s18);
  for (int d = 0; d < 3; ++d) sizes.push_back((size_t)NS * g.fl1[d].cells() * sizeof(double));
  for (int d1 = 0; d1 < 3; ++d1)
    for (int d2 = 0; d2 < 3; ++d2)
      if (d1 != d2) sizes.push_back((size_t)NS * g.fl1[d1].cells() * sizeof(double));
  for (int d = 0; d < 3; ++d) sizes.push_back((size_t)NS * g.flF[d].cells() * sizeof(double));
  sizes.push_back(2 * (size_t)g.fplane.cells() * sizeof(double));
  for (int k = 0; k < 3; ++k) sizes.push_back((size_t)TMK_NCOMP * g.fplane.cells() * sizeof(double));
  size_t total = 0;
  for (size_t z : sizes) total += align_up3(z);
  cudaStream_t s = (cudaStream_t)stream;
  if (total > c->scratch_bytes) {
    TMK_CU(cudaStreamSynchronize(s));
    cudaFree(c->scratch);
    c->scratch = nullptr; c->scratch_bytes = 0;
    if (cudaMalloc(&c->scratch, total) != cudaSuccess) return TMK_ERR_ALLOC;
    c->scratch_bytes = total;
  }
  char* base = (char*)c->scratch;
  size_t off = 0, n = 0;
  auto take = [&]() { double* p = (double*)(base + off); off += align_up3(sizes[n++]); return p; };
  for (int d = 0; d < 3; ++d) g.WM[d] = take();
  for (int d = 0; d < 3; ++d) g.WP[d] = take();
  for (int d = 0; d < 3; ++d) g.WH1[d] = take();
  for (int d1 = 0; d1 < 3; ++d1)
    for (int d2 = 0; d2 < 3; ++d2)
      if (d1 != d2) g.WH2[d1][d2] = take();
  for (int d = 0; d < 3; ++d) g.WH[d] = take();
  g.LG = take();
  for (int k = 0; k < 3; ++k) g.FF[k] = take();

  const tmk::DevParams* P = c->dp;
  tmk::DevStatus* st = c->dstatus;
  const unsigned bS = blocks(g.S.cells());
  pred_kernel<0><<<bS, 128, 0, s>>>(g, P);
  pred_kernel<1><<<bS, 128, 0, s>>>(g, P);
  pred_kernel<2><<<bS, 128, 0, s>>>(g, P);
  riem1_kernel<0><<<blocks(g.fl1[0].cells()), 128, 0, s>>>(g, P, st);
  riem1_kernel<1><<<blocks(g.fl1[1].cells()), 128, 0, s>>>(g, P, st);
  riem1_kernel<2><<<blocks(g.fl1[2].cells()), 128, 0, s>>>(g, P, st);
  riem2_kernel<0, 1><<<blocks(g.fl1[0].cells()), 128, 0, s>>>(g, P, st);
  riem2_kernel<0, 2><<<blocks(g.fl1[0].cells()), 128, 0, s>>>(g, P, st);
  riem2_kernel<1, 0><<<blocks(g.fl1[1].cells()), 128, 0, s>>>(g, P, st);
  riem2_kernel<1, 2><<<blocks(g.fl1[1].cells()), 128, 0, s>>>(g, P, st);
  riem2_kernel<2, 0><<<blocks(g.fl1[2].cells()), 128, 0, s>>>(g, P, st);
  riem2_kernel<2, 1><<<blocks(g.fl1[2].cells()), 128, 0, s>>>(g, P, st);
  final_kernel<0><<<blocks(g.flF[0].cells()), 128, 0, s>>>(g, P, st);
  final_kernel<1><<<blocks(g.flF[1].cells()), 128, 0, s>>>(g, P, st);
  final_kernel<2><<<blocks(g.flF[2].cells()), 128, 0, s>>>(g, P, st);
  if (g.F[0]) flux_kernel<0><<<blocks(g.flF[0].cells()), 128, 0, s>>>(g, P);
  if (g.F[1]) flux_kernel<1><<<blocks(g.flF[1].cells()), 128, 0, s>>>(g, P);
  if (g.F[2]) flux_kernel<2><<<blocks(g.flF[2].cells()), 128, 0, s>>>(g, P);
  update_kernel<<<blocks(cur.cells()), 128, 0, s>>>(g, P);
  if (g.fault) bdry_final_kernel<<<blocks((long long)cur.n[0] * cur.n[2]), 128, 0, s>>>(g, P, st);
  TMK_CU(cudaGetLastError());
  if (max_wave_speed) *max_wave_speed = std::max(c->hp.cs, c->hp.cp);
  return TMK_OK;
}

extern "C" tmk_status tmk_plastic_update_3d(tmk_context* c, const tmk_fab3* U, const tmk_box3* box, double dt,
                                            void* stream) {
  if (!c || !U || !U->data || !box || U->ncomp != TMK_NCOMP) return TMK_ERR_BAD_DESC;
  const Bx A = bx_of(U->lo, U->hi), b = bx_of(box->lo, box->hi);
  if (!bx_ok(A) || !bx_ok(b) || !bx_contains(A, b)) return TMK_ERR_BAD_DESC;
  tmk::d3::plastic3_kernel<<<tmk::d3::blocks(b.cells()), 128, 0, (cudaStream_t)stream>>>(U->data, A, b, c->dp, dt);
  TMK_CU(cudaGetLastError());
  return TMK_OK;
}
