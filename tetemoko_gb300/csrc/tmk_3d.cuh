// The 3-D patch step (CH_SPACEDIM == 3): kernels, templated on the arithmetic
// of the volume stencil T.
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
//                were moved by -(1/3) dt/dx A dW/dx of WHalf1[D2] (:329-381);
//                both D2 of a D1 in one pass (riem2_pair) that reads the
//                normal states once
//   final<D1>    the time-centred WHalf[D1], normal states moved by both
//                WHalf2[D2][D3] with -(1/2) dt/dx (:422-440)
//   update       fluxes, their divergence and U += -dt/dx dU in place; then
//                the fault's boundary data (RSSETBND / SWSETBND, final)
// Cell states (WM, WP) and face states are stored with the 12 components that
// the transverse terms and the fluxes read.
// The fault is the y-lo plane of the domain.  Its boundary data predicted at
// (1/3) dt from WHalf1[1] and at (1/2) dt from WHalf2[1][2] (the reference's
// call order leaves those in m_tmpBdryData when WHalf2[1][*] and WHalf[1] are
// solved) are formed at the face that reads them.  Fault faces keep all 22
// components of their states (FP64) beside the 18-component arrays, because
// the reference-layout slip-weakening law reads and writes side 2 from
// component 9.
//
// T = double: the plain FP64 form (built without FMA contraction; equal to the
// CPU oracle to rounding).  T = float: the mixed form -- predictors, Riemann
// solves, transverse corrections and fluxes in FP32 with FP32 intermediates;
// the state U, its update, the friction solves (the 2-D mixed form's
// arrangement for rate and state) and the boundary data in FP64.
#pragma once

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
  // t < cells() < 2^31 (every box of a step lies in the nodes of U's box,
  // whose node count the host keeps below 2^31): 32-bit unsigned division,
  // several times cheaper on the GPU than the 64-bit one.
  TMK_HD void cell(long long t, int& i, int& j, int& k) const {
    const unsigned u = (unsigned)t, n0 = (unsigned)n[0], n1 = (unsigned)n[1];
    const unsigned r = u / n0, q = r / n1;
    i = lo[0] + (int)(u - r * n0);
    j = lo[1] + (int)(r - q * n1);
    k = lo[2] + (int)q;
  }
};

template <typename T>
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
  T* WM[3];
  T* WP[3];
  T* WH1[3];
  T* WH2[3][3];         // WHalf2[d1][d2], d1 != d2
  T* WH[3];
  double* LG;           // lambda, gamma of side 1 predicted at the fault's lo faces (fplane)
  double* FF[3];        // 22-comp fault-face states of WHalf1[1], WHalf2[1][2], WHalf[1] (fplane)
  double* B;
  double* F[3];         // optional face fluxes (22 comps over flF[d])
  double dx, dt, time;
  int fault;
  // the predictors' input: U itself (FP64 form; side s at component 11 s) or
  // its FP32 copy over grow(valid, 3) & domain made once per step (mixed form;
  // side s at component 9 s), so that no predictor converts FP64 values
  const T* Up;
  T* Uc;                // the FP32 copy (mixed form; Up == Uc), else null
  Bx Ap;
  int uside;
  Consts<T> kc;         // the physical constants in T (computed on the host)
  T sig[NSIDE];         // characteristic Courant numbers lambda dt/dx
  T scale3, scale2;     // -(1/3) dt/dx and -(1/2) dt/dx
  double sc;            // -dt/dx
  // mixed form, PPM with primitive limiting: the branch-free predictor
  // with these tracing coefficients
  int fastpred;
  T trA[NSIDE], trB[NSIDE];
};

template <int D> TMK_HD double rvs(int s) { return (D == 1 && s == 1) ? -1.0 : 1.0; }

// States of direction D are stored with the components the transverse terms
// (adwdx_add) and the fluxes read from its face states: the rotated cx, cy, cz,
// cx+3, cxy, cxz of each side (12 of 18).  These face components come from the
// same components of the cell states (RIEMANNF and the edge conditions form
// them from the waves sxx -/+ Zp vx, sxy -/+ Zs vy, sxz -/+ Zs vz), and the
// fault laws' outputs that anything reads (the face state's velocities, syy,
// sxy, syz and the boundary data) depend on those components of the interior
// state only; so the normal states WM/WP of direction D are stored with the
// same 12 components, and the predictor's work for the other three (the
// zero-speed waves wyy, wzz, wyz) is dropped by the compiler.  Fault faces keep
// all 22 components of their states in FF.
constexpr int NF = 12;
template <int D> TMK_D constexpr int face_comp(int m) {
  using R = Rot<D>;
  return m == 0 ? R::cx : m == 1 ? R::cy : m == 2 ? R::cz : m == 3 ? R::cx + 3 : m == 4 ? R::cxy : R::cxz;
}
template <int D, typename T>
TMK_D void store_face(T* a, const Bx& b, int i, int j, int k, const T* q) {
  const long long cs = b.cells(), o = b.at(i, j, k);
#pragma unroll
  for (int s = 0; s < 2; ++s)
#pragma unroll
    for (int m = 0; m < 6; ++m) a[(6 * s + m) * cs + o] = q[NSIDE * s + face_comp<D>(m)];
}
template <int D, typename T>
TMK_D void load_face(const T* a, const Bx& b, int i, int j, int k, T* q) {
  const long long cs = b.cells(), o = b.at(i, j, k);
#pragma unroll
  for (int c = 0; c < NS; ++c) q[c] = T(0);
#pragma unroll
  for (int s = 0; s < 2; ++s)
#pragma unroll
    for (int m = 0; m < 6; ++m) q[NSIDE * s + face_comp<D>(m)] = a[(6 * s + m) * cs + o];
}

template <int D> TMK_D void step(int& i, int& j, int& k, int s) {
  if (D == 0) i += s; else if (D == 1) j += s; else k += s;
}
template <int D> TMK_D int coord(int i, int j, int k) { return D == 0 ? i : (D == 1 ? j : k); }

// Face t of the y-face box fb with the fault plane (its first y layer) first:
// the friction solves, long chains of dependent FP64 operations, then start
// with the grid and run beside the bulk instead of trailing it.
TMK_D void face_fault_first(const Bx& fb, bool fault, long long t, int& i, int& j, int& k) {
  if (!fault) { fb.cell(t, i, j, k); return; }
  const unsigned nx = (unsigned)fb.n[0], nf = nx * (unsigned)fb.n[2];
  unsigned u = (unsigned)t;
  if (u < nf) {
    const unsigned q = u / nx;
    i = fb.lo[0] + (int)(u - q * nx);
    j = fb.lo[1];
    k = fb.lo[2] + (int)q;
    return;
  }
  u -= nf;
  const unsigned ny = (unsigned)fb.n[1] - 1, r = u / nx, q = r / ny;
  i = fb.lo[0] + (int)(u - r * nx);
  j = fb.lo[1] + 1 + (int)(r - q * ny);
  k = fb.lo[2] + (int)q;
}
template <int D> TMK_D void face_at(const Bx& fb, bool fault, long long t, int& i, int& j, int& k) {
  if (D == 1) face_fault_first(fb, fault, t, i, j, k);
  else fb.cell(t, i, j, k);
}

// Which faces a launch of a face pass covers: all of them, the bulk (the
// fault plane excluded) or the fault plane alone.  The fault plane's passes
// run on a second stream beside the bulk (launch_plan).
enum : int { PART_ALL = 0, PART_BULK = 1, PART_FAULT = 2 };
template <int D>
TMK_HD long long part_faces(const Bx& fb, bool fault, int part) {
  const long long nf = (D == 1 && fault) ? (long long)fb.n[0] * fb.n[2] : 0;
  return part == PART_BULK ? fb.cells() - nf : part == PART_FAULT ? nf : fb.cells();
}
// face t of a launch covering `part` (t < part_faces)
template <int D>
TMK_D void part_face(const Bx& fb, bool fault, int part, long long t, int& i, int& j, int& k) {
  if (D == 1 && fault && part == PART_BULK) t += (long long)fb.n[0] * fb.n[2];
  face_at<D>(fb, fault, t, i, j, k);
}

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
// ------------------------------------------------------ work of a launch
// A launch covers one patch (its descriptor passed by value) or the patches of
// a batch (descriptors in device memory, with the prefix sums of the pass's
// work per patch): find() gives thread t's patch and its index there.
template <typename T>
struct One {
  Step3<T> g;
  TMK_D const Step3<T>* find(long long t, long long& lt) const { lt = t; return &g; }
};
template <typename T>
struct Many {
  const Step3<T>* gs;
  const long long* start;   // np + 1 prefix sums of the pass's work
  int np;
  TMK_D const Step3<T>* find(long long t, long long& lt) const {
    if (t >= start[np]) return nullptr;
    int lo = 0, hi = np - 1;            // the last patch whose work starts at or before t
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (start[mid] <= t) lo = mid; else hi = mid - 1;
    }
    lt = t - start[lo];
    return gs + lo;
  }
};
#define TMK3_FIND(T)                                                                 \
  long long lt;                                                                      \
  const Step3<T>* gp = src.find(blockIdx.x * (long long)blockDim.x + threadIdx.x, lt); \
  if (!gp) return;

// The slope box halved along D: each pred thread takes two neighbouring cells
// along D (the last one alone where the box has odd length), whose PPM
// stencils share four of their five points.
template <int D> TMK_HD Bx pair_box(const Bx& S) {
  Bx b = S;
  b.n[D] = (S.n[D] + 1) / 2;
  return b;
}

template <int D, typename T>
TMK_D void pred_body(const Step3<T>& g, const DevParams& P, long long t) {
  const Bx pb = pair_box<D>(g.S);
  if (t >= pb.cells()) return;
  int i, j, k;
  pb.cell(t, i, j, k);
  if (D == 0) i = g.S.lo[0] + 2 * (i - g.S.lo[0]);
  else if (D == 1) j = g.S.lo[1] + 2 * (j - g.S.lo[1]);
  else k = g.S.lo[2] + 2 * (k - g.S.lo[2]);
  const Consts<T>& kc = g.kc;
  const T* sig = g.sig;
  const int q0 = coord<D>(i, j, k);
  const bool two = q0 + 1 < g.S.lo[D] + g.S.n[D];
  // window points q0-2 .. q0+3; the last is read only for a second cell (the
  // predictor input covers the slope box grown by 2 within the domain)
  bool in[6];
#pragma unroll
  for (int m = 0; m < 6; ++m) in[m] = q0 - 2 + m >= g.dlo[D] && q0 - 2 + m <= g.dhi[D];
  in[5] = in[5] && two;
  const long long acs = g.A.cells(), pcs = g.Ap.cells();
  T WM0[NS], WP0[NS], WM1[NS], WP1[NS];
#pragma unroll
  for (int s = 0; s < 2; ++s) {
    T w6[NSIDE][6];
#pragma unroll
    for (int m = 0; m < 6; ++m) {
      int ii = i, jj = j, kk = k;
      step<D>(ii, jj, kk, m - 2);
      const long long o = in[m] ? g.Ap.at(ii, jj, kk) : 0;
#pragma unroll
      for (int c = 0; c < NSIDE; ++c) w6[c][m] = in[m] ? g.Up[(g.uside * s + c) * pcs + o] : T(0);
    }
    bool fast = false;
    if constexpr (!kExact<T>) fast = g.fastpred != 0;
    if (fast) {
      ppm_predict_prim2<D, T>(kc, (T)rvs<D>(s), w6, in, two, g.trA, g.trB, WM0 + NSIDE * s, WP0 + NSIDE * s,
                              WM1 + NSIDE * s, WP1 + NSIDE * s);
    } else {
      T w5[NSIDE][5];
#pragma unroll
      for (int c = 0; c < NSIDE; ++c)
#pragma unroll
        for (int m = 0; m < 5; ++m) w5[c][m] = w6[c][m];
      ppm_predict<D, T>(kc, (T)rvs<D>(s), w5, in, P.prim_lim != 0, P.char_lim != 0, sig, WM0 + NSIDE * s,
                        WP0 + NSIDE * s, P.order, P.fourth != 0);
      if (two) {
#pragma unroll
        for (int c = 0; c < NSIDE; ++c)
#pragma unroll
          for (int m = 0; m < 5; ++m) w5[c][m] = w6[c][m + 1];
        ppm_predict<D, T>(kc, (T)rvs<D>(s), w5, in + 1, P.prim_lim != 0, P.char_lim != 0, sig, WM1 + NSIDE * s,
                          WP1 + NSIDE * s, P.order, P.fourth != 0);
      }
    }
  }
  store_face<D>(g.WM[D], g.S, i, j, k, WM0);
  store_face<D>(g.WP[D], g.S, i, j, k, WP0);
  if (two) {
    int i1 = i, j1 = j, k1 = k;
    step<D>(i1, j1, k1, 1);
    store_face<D>(g.WM[D], g.S, i1, j1, k1, WM1);
    store_face<D>(g.WP[D], g.S, i1, j1, k1, WP1);
  }
  if (D == 1 && g.fault && j == g.dlo[1]) {
    // lambda and gamma of side 1 at the fault's lo faces (read by the
    // reference-layout slip-weakening law as side-2 velocities); only the
    // first cell of a pair can lie on the domain's y-lo layer
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
template <int D, typename T, typename Src>
__global__ void __launch_bounds__(128) pred_kernel(const __grid_constant__ Src src, const DevParams* Pp) {
  TMK3_FIND(T)
  pred_body<D, T>(*gp, *Pp, lt);
}

// -------------------------------------------------------- face conditions
// Boundary data value the fault law reads at face (i, k): psi (rate and
// state) or slip (slip weakening), from B, or from B moved by the 22-comp face
// state U22 over `dtp` (the predictor's m_tmpBdryData, updateBoundary final=false).
template <typename T>
TMK_D double bdry_value(const DevParams& P, const Step3<T>& g, int i, int k, const double* U22, double dtp) {
  double* Bi = g.B + g.bb.at(i, g.dlo[1], k);
  const long long bs = g.bb.cells();
  if (!U22) return P.fault_law == 1 ? Bi[10 * bs] : Bi[7 * bs];
  if (P.fault_law == 1) {
    const RSFace fr = rs_face(P, nullptr, 0, 0);
    const double x = (i + 0.5) * g.dx - P.rs_x0;
    if constexpr (!kExact<T>) return rs_setbnd_k(P, rs_face_k(P, fr, x), U22, Bi, (int)bs, dtp, 0.0, false);
    return rs_setbnd(P, fr, U22, Bi, (int)bs, dtp, x, 0.0, false);
  }
  return sw_setbnd(P, U22, Bi, (int)bs, dtp, 0.0, false);
}

// fault face (i, dom lo, k): 22-comp state Wg from the interior state Wi22.
// The mixed form solves the rate-and-state friction equation with the
// latency-arranged z-space Newton of the 2-D mixed form (rs_fault_k): the
// 3-D law is the 2-D one (no antiplane characteristic, nucleation in x).
template <typename T>
TMK_D void fault_face(const DevParams& P, double dx, int i, int k, const double* Wi, double bval, double* Wg,
                      DevStatus* st) {
#pragma unroll
  for (int c = 0; c < NC; ++c) Wg[c] = 0.0;
  const double xc = (i + 0.5) * dx;
  if (P.fault_law == 1) {
    const RSFace fr = rs_face(P, nullptr, 0, 0);
    int it;
    if constexpr (!kExact<T>) it = rs_fault_k(P, rs_face_k(P, fr, xc - P.rs_x0), Wi, bval, Wg);
    else it = rs_fault(P, fr, Wi, bval, xc - P.rs_x0, Wg);
    if (it > RS_IMAX) atomicAdd(&st->newton_maxed, 1ull);
  } else {
    sw_fault<true>(P, Wi, bval, xc, Wg, (k + 0.5) * dx);
  }
}

// Face f of direction D with left cell state L18 and right cell state R18:
// Riemann solve, or the domain-edge condition.  Returns false for the fault
// faces (y lo with a fault law), which the caller solves.
template <int D, typename T>
TMK_D bool face_state(const DevParams& P, const Consts<T>& kc, const Step3<T>& g, int f, const T* L18,
                      const T* R18, T* G18) {
  if (f == g.dlo[D] || f == g.dhi[D] + 1) {
    const bool lo = f == g.dlo[D];
    if (lo && D == 1 && g.fault) return false;
    const bool outflow = P.bc[2 * D + (lo ? 0 : 1)] == 0;
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      // the interior state by element-wise selects (a select of the array
      // pointer would put both arrays in local memory)
      T bg[NSIDE], wi[NSIDE];
#pragma unroll
      for (int c = 0; c < NSIDE; ++c) {
        bg[c] = (T)P.bg[11 * s + c];
        wi[c] = lo ? R18[NSIDE * s + c] : L18[NSIDE * s + c];
      }
      edge_bc<D, T>(kc, (T)rvs<D>(s), lo ? -1 : +1, outflow, bg, wi, G18 + NSIDE * s);
    }
  } else {
#pragma unroll
    for (int s = 0; s < 2; ++s) riemann<D, T>(kc, (T)rvs<D>(s), L18 + NSIDE * s, R18 + NSIDE * s, G18 + NSIDE * s);
  }
  return true;
}

// fault face: gather the 22-comp interior state, solve in FP64, keep 22 comps in FFk
template <typename T>
TMK_D void fault_solve(const DevParams& P, const Step3<T>& g, int i, int k, const T* R18, double bval,
                       double* FFk, T* G18, DevStatus* st) {
  double Wi[NC], Wg[NC];
  const long long fo = g.fplane.at(i, g.dlo[1], k), fcs = g.fplane.cells();
#pragma unroll
  for (int c = 0; c < NSIDE; ++c) { Wi[c] = (double)R18[c]; Wi[11 + c] = (double)R18[NSIDE + c]; }
  Wi[9] = g.LG[fo]; Wi[10] = g.LG[fcs + fo];
  Wi[20] = 0.0; Wi[21] = 0.0;
  fault_face<T>(P, g.dx, i, k, Wi, bval, Wg, st);
#pragma unroll
  for (int c = 0; c < NSIDE; ++c) { G18[c] = (T)Wg[c]; G18[NSIDE + c] = (T)Wg[11 + c]; }
  if (FFk) {
#pragma unroll
    for (int c = 0; c < NC; ++c) FFk[c * fcs + fo] = Wg[c];
  }
}

template <typename T>
TMK_D void load_ff(const Step3<T>& g, const double* FFk, int i, int k, double* U22) {
  const long long fo = g.fplane.at(i, g.dlo[1], k), fcs = g.fplane.cells();
#pragma unroll
  for (int c = 0; c < NC; ++c) U22[c] = FFk[c * fcs + fo];
}

// ------------------------------------------------------------ first pass
// FC = false: a launch without fault faces (the bulk part), built without the
// friction solve's code and registers.
template <int D, typename T, bool FC = true>
TMK_D void riem1_body(const Step3<T>& g, const DevParams& P, DevStatus* st, int part, long long t) {
  const Bx& fb = g.fl1[D];
  if (t >= part_faces<D>(fb, g.fault != 0, part)) return;
  int i, j, k;
  part_face<D>(fb, g.fault != 0, part, t, i, j, k);
  const Consts<T>& kc = g.kc;
  const int f = coord<D>(i, j, k);
  T L[NS], R[NS], G[NS];
  int li = i, lj = j, lk = k;
  step<D>(li, lj, lk, -1);
  if (f > g.dlo[D]) load_face<D>(g.WP[D], g.S, li, lj, lk, L);
  if (f <= g.dhi[D]) load_face<D>(g.WM[D], g.S, i, j, k, R);
  if (!face_state<D, T>(P, kc, g, f, L, R, G)) {
    if constexpr (FC) fault_solve(P, g, i, k, R, bdry_value(P, g, i, k, nullptr, 0.0), g.FF[0], G, st);
  }
  store_face<D>(g.WH1[D], fb, i, j, k, G);
}
template <int D, typename T, typename Src, bool FC = true>
__global__ void __launch_bounds__(128) riem1_kernel(const __grid_constant__ Src src, const DevParams* Pp,
                                                    DevStatus* st, int part) {
  TMK3_FIND(T)
  riem1_body<D, T, FC>(*gp, *Pp, st, part, lt);
}

// cell state T18 (direction-D1 normal states) at (i, j, k) moved by -(scale)
// A dW/dx of the face states H in direction D2 where the cell lies in ccBox[D2]
template <int D2, typename T>
TMK_D void add_transverse(const Step3<T>& g, const Consts<T>& kc, const T* H, const Bx& hb, T scale, int i, int j,
                          int k, T* T18) {
  if (!g.cc[D2].has(i, j, k)) return;
  T h[NS], l[NS];
  int hi = i, hj = j, hk = k;
  step<D2>(hi, hj, hk, 1);
  load_face<D2>(H, hb, hi, hj, hk, h);
  load_face<D2>(H, hb, i, j, k, l);
#pragma unroll
  for (int s = 0; s < 2; ++s)
    adwdx_add<D2, T>(kc, (T)rvs<D2>(s), scale, h + NSIDE * s, l + NSIDE * s, T18 + NSIDE * s);
}

// ----------------------------------------------------------- second pass
// The normal states WP[D1] of the left and WM[D1] of the right cell of the D1
// face (i, j, k), where those cells lie in the domain.
template <int D1, typename T>
TMK_D void riem2_load(const Step3<T>& g, int i, int j, int k, bool hasL, bool hasR, T* L0, T* R0) {
  int li = i, lj = j, lk = k;
  step<D1>(li, lj, lk, -1);
  if (hasL) load_face<D1>(g.WP[D1], g.S, li, lj, lk, L0);
  if (hasR) load_face<D1>(g.WM[D1], g.S, i, j, k, R0);
}

// WHalf2[D1][D2] at the D1 face (i, j, k) from the normal states L0, R0 of its
// two cells: the transverse corrections of WHalf1[D2], then the Riemann solve
// or the face's condition.
template <int D1, int D2, typename T, bool FC = true>
TMK_D void riem2_solve(const Step3<T>& g, const DevParams& P, DevStatus* st, int i, int j, int k, bool hasL,
                       bool hasR, const T* L0, const T* R0) {
  const Consts<T>& kc = g.kc;
  const T scale = g.scale3;
  T L[NS], R[NS], G[NS];
  if (hasL) {
    int li = i, lj = j, lk = k;
    step<D1>(li, lj, lk, -1);
#pragma unroll
    for (int c = 0; c < NS; ++c) L[c] = L0[c];
    add_transverse<D2, T>(g, kc, g.WH1[D2], g.fl1[D2], scale, li, lj, lk, L);
  }
  if (hasR) {
#pragma unroll
    for (int c = 0; c < NS; ++c) R[c] = R0[c];
    add_transverse<D2, T>(g, kc, g.WH1[D2], g.fl1[D2], scale, i, j, k, R);
  }
  if (!face_state<D1, T>(P, kc, g, coord<D1>(i, j, k), L, R, G)) {
    if constexpr (!FC) return;
    double U22[NC];
    load_ff(g, g.FF[0], i, k, U22);
    const double bval = bdry_value(P, g, i, k, U22, (1.0 / 3.0) * g.dt);
    fault_solve(P, g, i, k, R, bval, (D2 == 2) ? g.FF[1] : nullptr, G, st);
  }
  store_face<D1>(g.WH2[D1][D2], g.fl1[D1], i, j, k, G);
}

template <int D1, int D2, typename T>
TMK_D void riem2_face(const Step3<T>& g, const DevParams& P, DevStatus* st, int part, long long t) {
  const Bx& fb = g.fl1[D1];
  if (t >= part_faces<D1>(fb, g.fault != 0, part)) return;
  int i, j, k;
  part_face<D1>(fb, g.fault != 0, part, t, i, j, k);
  const int f = coord<D1>(i, j, k);
  const bool hasL = f > g.dlo[D1], hasR = f <= g.dhi[D1];
  T L0[NS], R0[NS];
  riem2_load<D1, T>(g, i, j, k, hasL, hasR, L0, R0);
  riem2_solve<D1, D2, T>(g, P, st, i, j, k, hasL, hasR, L0, R0);
}

// WHalf2[D1][Da] and WHalf2[D1][Db] (Da, Db the other two directions) at a D1
// face, the normal states read once for both
template <int D1, typename T, bool FC>
TMK_D void riem2_pair_face(const Step3<T>& g, const DevParams& P, DevStatus* st, int part, long long t) {
  constexpr int Da = D1 == 0 ? 1 : 0, Db = D1 == 2 ? 1 : 2;
  const Bx& fb = g.fl1[D1];
  if (t >= part_faces<D1>(fb, g.fault != 0, part)) return;
  int i, j, k;
  part_face<D1>(fb, g.fault != 0, part, t, i, j, k);
  const int f = coord<D1>(i, j, k);
  const bool hasL = f > g.dlo[D1], hasR = f <= g.dhi[D1];
  T L0[NS], R0[NS];
  riem2_load<D1, T>(g, i, j, k, hasL, hasR, L0, R0);
  riem2_solve<D1, Da, T, FC>(g, P, st, i, j, k, hasL, hasR, L0, R0);
  riem2_solve<D1, Db, T, FC>(g, P, st, i, j, k, hasL, hasR, L0, R0);
}

template <int D1, typename T, typename Src, bool FC = true>
__global__ void __launch_bounds__(128) riem2_pair_kernel(const __grid_constant__ Src src, const DevParams* Pp,
                                                         DevStatus* st, int part) {
  TMK3_FIND(T)
  riem2_pair_face<D1, T, FC>(*gp, *Pp, st, part, lt);
}

// WHalf2[1][0] and WHalf2[1][2] on the fault plane in one launch (grid y = 0,
// 1): the two friction solves of a face run side by side
template <typename T, typename Src>
__global__ void __launch_bounds__(128) riem2_fault_kernel(const __grid_constant__ Src src, const DevParams* Pp,
                                                          DevStatus* st) {
  TMK3_FIND(T)
  if (blockIdx.y == 0) riem2_face<1, 0, T>(*gp, *Pp, st, PART_FAULT, lt);
  else riem2_face<1, 2, T>(*gp, *Pp, st, PART_FAULT, lt);
}

// ------------------------------------------------------------ final pass
template <int D1, int Dc, typename T>
TMK_D void add_final(const Step3<T>& g, const Consts<T>& kc, T scale, int i, int j, int k, T* T18) {
  if (!g.cc[Dc].has(i, j, k)) return;
  constexpr int D3 = 3 - D1 - Dc;
  T h[NS], l[NS];
  int hi = i, hj = j, hk = k;
  step<Dc>(hi, hj, hk, 1);
  load_face<Dc>(g.WH2[Dc][D3], g.fl1[Dc], hi, hj, hk, h);
  load_face<Dc>(g.WH2[Dc][D3], g.fl1[Dc], i, j, k, l);
#pragma unroll
  for (int s = 0; s < 2; ++s)
    adwdx_add<Dc, T>(kc, (T)rvs<Dc>(s), scale, h + NSIDE * s, l + NSIDE * s, T18 + NSIDE * s);
}

template <int D1, typename T>
TMK_D void final_state(const Step3<T>& g, const Consts<T>& kc, const T* A, T scale, int i, int j, int k, T* T18) {
  constexpr int Da = (D1 == 0) ? 1 : 0;      // the two other directions, ascending
  constexpr int Db = (D1 == 2) ? 1 : 2;
  load_face<D1>(A, g.S, i, j, k, T18);
  add_final<D1, Da, T>(g, kc, scale, i, j, k, T18);
  add_final<D1, Db, T>(g, kc, scale, i, j, k, T18);
}

template <int D1, typename T, bool FC>
TMK_D void final_body(const Step3<T>& g, const DevParams& P, DevStatus* st, int part, long long t) {
  const Bx& fb = g.flF[D1];
  if (t >= part_faces<D1>(fb, g.fault != 0, part)) return;
  int i, j, k;
  part_face<D1>(fb, g.fault != 0, part, t, i, j, k);
  const Consts<T>& kc = g.kc;
  const T scale = g.scale2;
  const int f = coord<D1>(i, j, k);
  T L[NS], R[NS], G[NS];
  int li = i, lj = j, lk = k;
  step<D1>(li, lj, lk, -1);
  if (f > g.dlo[D1]) final_state<D1, T>(g, kc, g.WP[D1], scale, li, lj, lk, L);
  if (f <= g.dhi[D1]) final_state<D1, T>(g, kc, g.WM[D1], scale, i, j, k, R);
  if (!face_state<D1, T>(P, kc, g, f, L, R, G)) {
    if constexpr (!FC) return;
    double U22[NC];
    load_ff(g, g.FF[1], i, k, U22);
    const double bval = bdry_value(P, g, i, k, U22, (1.0 / 2.0) * g.dt);
    fault_solve(P, g, i, k, R, bval, g.FF[2], G, st);
  }
  store_face<D1>(g.WH[D1], fb, i, j, k, G);
}
template <int D1, typename T, typename Src, bool FC = true>
__global__ void __launch_bounds__(128) final_kernel(const __grid_constant__ Src src, const DevParams* Pp,
                                                    DevStatus* st, int part) {
  TMK3_FIND(T)
  final_body<D1, T, FC>(*gp, *Pp, st, part, lt);
}

// ---------------------------------------------------------------- update
template <int D, typename T>
TMK_D void flux_diff(const Step3<T>& g, const Consts<T>& kc, int i, int j, int k, T* dU) {
  T h[NS], l[NS], Fh[NS], Fl[NS];
  int hi = i, hj = j, hk = k;
  step<D>(hi, hj, hk, 1);
  load_face<D>(g.WH[D], g.flF[D], hi, hj, hk, h);
  load_face<D>(g.WH[D], g.flF[D], i, j, k, l);
#pragma unroll
  for (int s = 0; s < 2; ++s) {
    flux<D, T>(kc, (T)rvs<D>(s), h + NSIDE * s, Fh + NSIDE * s);
    flux<D, T>(kc, (T)rvs<D>(s), l + NSIDE * s, Fl + NSIDE * s);
  }
#pragma unroll
  for (int c = 0; c < NS; ++c) dU[c] += Fh[c] - Fl[c];
}

template <typename T>
TMK_D void update_body(const Step3<T>& g, long long t) {
  if (t >= g.cur.cells()) return;
  int i, j, k;
  g.cur.cell(t, i, j, k);
  const Consts<T>& kc = g.kc;
  T dU[NS];
#pragma unroll
  for (int c = 0; c < NS; ++c) dU[c] = T(0);
  flux_diff<0, T>(g, kc, i, j, k, dU);
  flux_diff<1, T>(g, kc, i, j, k, dU);
  flux_diff<2, T>(g, kc, i, j, k, dU);
  const double sc = g.sc;
  const long long acs = g.A.cells(), o = g.A.at(i, j, k);
#pragma unroll
  for (int s = 0; s < 2; ++s)
#pragma unroll
    for (int c = 0; c < NSIDE; ++c) {
      double* u = g.U + (11 * s + c) * acs + o;
      *u = *u + (double)dU[NSIDE * s + c] * sc;
    }
}
template <typename T, typename Src>
__global__ void __launch_bounds__(128) update_kernel(const __grid_constant__ Src src) {
  TMK3_FIND(T)
  update_body<T>(*gp, lt);
}

// the face fluxes of direction D (22 comps; lambda, gamma and the antiplane
// stress of the face normal carry none)
template <int D, typename T>
TMK_D void flux_body(const Step3<T>& g, long long t) {
  const Bx& fb = g.flF[D];
  if (t >= fb.cells() || !g.F[D]) return;
  int i, j, k;
  fb.cell(t, i, j, k);
  const Consts<T>& kc = g.kc;
  T w[NS], F[NS];
  load_face<D>(g.WH[D], fb, i, j, k, w);
#pragma unroll
  for (int s = 0; s < 2; ++s) flux<D, T>(kc, (T)rvs<D>(s), w + NSIDE * s, F + NSIDE * s);
  const long long cs = fb.cells();
  double* out = g.F[D] + t;
#pragma unroll
  for (int s = 0; s < 2; ++s) {
#pragma unroll
    for (int c = 0; c < NSIDE; ++c) out[(11 * s + c) * cs] = (double)F[NSIDE * s + c];
    out[(11 * s + 9) * cs] = 0.0;
    out[(11 * s + 10) * cs] = 0.0;
  }
}
template <int D, typename T, typename Src>
__global__ void __launch_bounds__(128) flux_kernel(const __grid_constant__ Src src) {
  TMK3_FIND(T)
  flux_body<D, T>(*gp, lt);
}

// the fault's boundary data, final (RSSETBND / SWSETBND over the valid x, z)
template <typename T>
TMK_D void bdry_final_body(const Step3<T>& g, const DevParams& P, DevStatus* st, long long t) {
  const int nx = g.cur.n[0], nz = g.cur.n[2];
  if (!g.fault || t >= (long long)nx * nz) return;
  const int i = g.cur.lo[0] + (int)(t % nx), k = g.cur.lo[2] + (int)(t / nx);
  double U22[NC];
  load_ff(g, g.FF[2], i, k, U22);
  const long long bo = g.bb.at(i, g.dlo[1], k);
  double* Bi = g.B + bo;
  const int bs = (int)g.bb.cells();
  if (P.fault_law == 1) {
    const RSFace fr = rs_face(P, nullptr, 0, 0);
    const double x = (i + 0.5) * g.dx - P.rs_x0;
    double psi;
    if constexpr (!kExact<T>) psi = rs_setbnd_k(P, rs_face_k(P, fr, x), U22, Bi, bs, g.dt, g.time + g.dt, true);
    else psi = rs_setbnd(P, fr, U22, Bi, bs, g.dt, x, g.time + g.dt, true);
    if (isnan(psi)) report(st, ST_NAN, bo);
  } else {
    sw_setbnd(P, U22, Bi, bs, g.dt, g.time + g.dt, true);
  }
}
template <typename T, typename Src>
__global__ void __launch_bounds__(128) bdry_final_kernel(const __grid_constant__ Src src, const DevParams* Pp,
                                                         DevStatus* st) {
  TMK3_FIND(T)
  bdry_final_body<T>(*gp, *Pp, st, lt);
}

// FP32 copy of the evolving components of U over Ap (mixed form)
template <typename T>
TMK_D void to_pred_body(const Step3<T>& g, long long t) {
  if (t >= g.Ap.cells()) return;
  T* out = g.Uc;
  int i, j, k;
  g.Ap.cell(t, i, j, k);
  const long long acs = g.A.cells(), o = g.A.at(i, j, k), pcs = g.Ap.cells();
#pragma unroll
  for (int s = 0; s < 2; ++s)
#pragma unroll
    for (int c = 0; c < NSIDE; ++c) out[(NSIDE * s + c) * pcs + t] = (T)g.U[(11 * s + c) * acs + o];
}
template <typename T, typename Src>
__global__ void __launch_bounds__(128) to_pred_kernel(const __grid_constant__ Src src) {
  TMK3_FIND(T)
  to_pred_body<T>(*gp, lt);
}

inline unsigned blocks(long long n) { return (unsigned)((n + 127) / 128); }

// ------------------------------------------------------------ work plans
// The work of each kind of pass: cells or faces, for the y-direction face
// passes also split into the bulk and the fault plane.
enum : int {
  K_AP = 0, K_SP0, K_SP1, K_SP2, K_FL1_0, K_FL1_1, K_FL1_1B, K_FL1_1F, K_FL1_2, K_FLF_0, K_FLF_1, K_FLF_1B, K_FLF_1F, K_FLF_2,
  K_CUR, K_BF, NKIND
};
template <typename T>
TMK_HD long long kind_count(const Step3<T>& g, int kind) {
  const bool f = g.fault != 0;
  switch (kind) {
    case K_AP: return g.Ap.cells();
    case K_SP0: return pair_box<0>(g.S).cells();
    case K_SP1: return pair_box<1>(g.S).cells();
    case K_SP2: return pair_box<2>(g.S).cells();
    case K_FL1_0: return g.fl1[0].cells();
    case K_FL1_1: return part_faces<1>(g.fl1[1], f, PART_ALL);
    case K_FL1_1B: return part_faces<1>(g.fl1[1], f, PART_BULK);
    case K_FL1_1F: return part_faces<1>(g.fl1[1], f, PART_FAULT);
    case K_FL1_2: return g.fl1[2].cells();
    case K_FLF_0: return g.flF[0].cells();
    case K_FLF_1: return part_faces<1>(g.flF[1], f, PART_ALL);
    case K_FLF_1B: return part_faces<1>(g.flF[1], f, PART_BULK);
    case K_FLF_1F: return part_faces<1>(g.flF[1], f, PART_FAULT);
    case K_FLF_2: return g.flF[2].cells();
    case K_CUR: return g.cur.cells();
    case K_BF: return f ? (long long)g.cur.n[0] * g.cur.n[2] : 0;
  }
  return 0;
}

// one patch: its descriptor by value
template <typename T>
struct PlanOne {
  using Src = One<T>;
  Step3<T> g;
  long long n(int kind) const { return kind_count(g, kind); }
  Src src(int) const { return Src{g}; }
  bool copy() const { return g.Up != (const T*)(const void*)g.U; }
  bool fault() const { return g.fault != 0; }
  bool flux(int d) const { return g.F[d] != nullptr; }
};
// a batch: descriptors and prefix sums in device memory, totals on the host
template <typename T>
struct PlanMany {
  using Src = Many<T>;
  const Step3<T>* dgs;
  const long long* dstart;     // NKIND x (np + 1)
  int np;
  long long tot[NKIND];
  bool copy_, fault_, flux_[3];
  long long n(int kind) const { return tot[kind]; }
  Src src(int kind) const { return Src{dgs, dstart + (size_t)kind * (np + 1), np}; }
  bool copy() const { return copy_; }
  bool fault() const { return fault_; }
  bool flux(int d) const { return flux_[d]; }
};

// Streams and events of the overlapped schedule (created with the context's
// first 3-D step)
struct Side {
  cudaStream_t s = nullptr;
  cudaEvent_t ev[6] = {};
};

// The whole step on stream s, for one patch or a batch.  When the work holds
// fault faces and a side stream is given, the three passes over the fault
// plane (their friction solves are chains of dependent FP64 operations) run on
// the side stream beside the bulk passes, forked and joined with events:
//   side: [pred<1>] F1 = riem1<1> fault | [riem1<0>, riem1<2>] F2 = riem2<1,0> and riem2<1,2> fault (one launch)
//         | [riem2<0,*>, riem2<2,*>] F3 = final<1> fault
//   main: pred x3, riem1<0>, riem1<2>, riem1<1> bulk, [F1] riem2<0,*>, riem2<2,*>, riem2<1,*> bulk,
//         final<1> bulk, [F2] final<0>, final<2>, [F3] update
// (riem2<D1,*>: WHalf2[D1][D2] for both D2 != D1 in one pass.)
// Each pass still reads exactly what the reference's order has written when
// it runs; the passes on the two streams write disjoint faces.
template <typename T, typename Plan>
cudaError_t launch_plan(const Plan& pl, const DevParams* P, DevStatus* st, cudaStream_t s, const Side* side) {
  using Src = typename Plan::Src;
  const bool split = pl.fault() && side && side->s;
  cudaStream_t fs = split ? side->s : s;
  const int bulk = split ? PART_BULK : PART_ALL;
  const int k11 = split ? K_FL1_1B : K_FL1_1, kf1 = split ? K_FLF_1B : K_FLF_1;
  auto fork = [&](int e) {
    if (!split) return;
    cudaEventRecord(side->ev[e], s);
    cudaStreamWaitEvent(fs, side->ev[e], 0);
  };
  auto join = [&](int e) {
    if (!split) return;
    cudaStreamWaitEvent(s, side->ev[e], 0);
  };
  auto nb = [&](int kind) { return blocks(pl.n(kind)); };
  if (pl.copy() && pl.n(K_AP)) to_pred_kernel<T, Src><<<nb(K_AP), 128, 0, s>>>(pl.src(K_AP));
  pred_kernel<0, T, Src><<<nb(K_SP0), 128, 0, s>>>(pl.src(K_SP0), P);
  pred_kernel<1, T, Src><<<nb(K_SP1), 128, 0, s>>>(pl.src(K_SP1), P);
  fork(0);
  if (split) {
    riem1_kernel<1, T, Src><<<nb(K_FL1_1F), 128, 0, fs>>>(pl.src(K_FL1_1F), P, st, PART_FAULT);
    cudaEventRecord(side->ev[3], fs);
  }
  pred_kernel<2, T, Src><<<nb(K_SP2), 128, 0, s>>>(pl.src(K_SP2), P);
  riem1_kernel<0, T, Src><<<nb(K_FL1_0), 128, 0, s>>>(pl.src(K_FL1_0), P, st, PART_ALL);
  riem1_kernel<2, T, Src><<<nb(K_FL1_2), 128, 0, s>>>(pl.src(K_FL1_2), P, st, PART_ALL);
  fork(1);
  if (split) {
    riem2_fault_kernel<T, Src><<<dim3(nb(K_FL1_1F), 2), 128, 0, fs>>>(pl.src(K_FL1_1F), P, st);
    cudaEventRecord(side->ev[4], fs);
  }
  if (split) riem1_kernel<1, T, Src, false><<<nb(k11), 128, 0, s>>>(pl.src(k11), P, st, bulk);
  else riem1_kernel<1, T, Src><<<nb(k11), 128, 0, s>>>(pl.src(k11), P, st, bulk);
  join(3);
  riem2_pair_kernel<0, T, Src><<<nb(K_FL1_0), 128, 0, s>>>(pl.src(K_FL1_0), P, st, PART_ALL);
  riem2_pair_kernel<2, T, Src><<<nb(K_FL1_2), 128, 0, s>>>(pl.src(K_FL1_2), P, st, PART_ALL);
  fork(2);
  if (split) {
    final_kernel<1, T, Src><<<nb(K_FLF_1F), 128, 0, fs>>>(pl.src(K_FLF_1F), P, st, PART_FAULT);
    cudaEventRecord(side->ev[5], fs);
  }
  if (split) riem2_pair_kernel<1, T, Src, false><<<nb(k11), 128, 0, s>>>(pl.src(k11), P, st, bulk);
  else riem2_pair_kernel<1, T, Src><<<nb(k11), 128, 0, s>>>(pl.src(k11), P, st, bulk);
  if (split) final_kernel<1, T, Src, false><<<nb(kf1), 128, 0, s>>>(pl.src(kf1), P, st, bulk);
  else final_kernel<1, T, Src><<<nb(kf1), 128, 0, s>>>(pl.src(kf1), P, st, bulk);
  join(4);
  final_kernel<0, T, Src><<<nb(K_FLF_0), 128, 0, s>>>(pl.src(K_FLF_0), P, st, PART_ALL);
  final_kernel<2, T, Src><<<nb(K_FLF_2), 128, 0, s>>>(pl.src(K_FLF_2), P, st, PART_ALL);
  join(5);
  if (pl.flux(0)) flux_kernel<0, T, Src><<<nb(K_FLF_0), 128, 0, s>>>(pl.src(K_FLF_0));
  if (pl.flux(1)) flux_kernel<1, T, Src><<<nb(K_FLF_1), 128, 0, s>>>(pl.src(K_FLF_1));
  if (pl.flux(2)) flux_kernel<2, T, Src><<<nb(K_FLF_2), 128, 0, s>>>(pl.src(K_FLF_2));
  update_kernel<T, Src><<<nb(K_CUR), 128, 0, s>>>(pl.src(K_CUR));
  if (pl.fault() && pl.n(K_BF)) bdry_final_kernel<T, Src><<<nb(K_BF), 128, 0, s>>>(pl.src(K_BF), P, st);
  return cudaGetLastError();
}

// FP64 instantiation (tmk_3d.cu, built without FMA contraction) and the mixed
// form (tmk_3d_f32.cu)
cudaError_t launch_one_f64(const PlanOne<double>& pl, const DevParams* P, DevStatus* st, cudaStream_t s,
                           const Side* side);
cudaError_t launch_many_f64(const PlanMany<double>& pl, const DevParams* P, DevStatus* st, cudaStream_t s,
                            const Side* side);
cudaError_t launch_one_f32(const PlanOne<float>& pl, const DevParams* P, DevStatus* st, cudaStream_t s,
                           const Side* side);
cudaError_t launch_many_f32(const PlanMany<float>& pl, const DevParams* P, DevStatus* st, cudaStream_t s,
                            const Side* side);

}  // namespace d3
}  // namespace tmk
