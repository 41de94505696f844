// tmk_kernels.cuh -- the device kernels of one level step, templated on the
// volume arithmetic type Real (double: plain FP64 form; float: mixed form).
//
//   fault_kernel   one thread per fault face (a warp per 32-face segment):
//                  predicts the two states that meet at the fault (rows 0-2 of
//                  the patch), runs the first-pass friction solve, the
//                  half-step state predictor, the transverse-corrected final
//                  solve and the boundary-data update, all friction work in FP64
//                  (LinElastPatchGodunov::computeWHalf call order,
//                  srcLinElast/LinElastPatchGodunov.cpp:289-452).
//   volume_kernel  one CTA per (tile, side): PPM normal predictors in x and y,
//                  first-pass Riemann, transverse corrections, final Riemann,
//                  fluxes and the conservative update (and, with plasticity,
//                  the Drucker-Prager return) of a TX x TY tile, every stage
//                  in shared memory; the fault faces come from fault_kernel.
//   exchange_kernel  same-level ghost copy between patches (LevelData::exchange).
#pragma once
#include "tmk_device.cuh"
#include "tmk_fault.cuh"

namespace tmk {

// One patch of a level on the device.
template <typename Real>
struct PatchDev {
  const Real* Uin;          // FAB over the allocated box, 22 component planes
  Real* Uout;
  int alo0, alo1, anx, any; // allocated box lo and extents
  int vlo0, vlo1, vhi0, vhi1;
  int dlo0, dlo1, dhi0, dhi1;
  double dx, dt;
  int scen;
  int plastic;              // apply the Drucker-Prager return after the update
  int fault;                // patch touches the y-lo fault
  double* B;                // fault FAB: nb planes over x in [blo0, blo0+bnx)
  int blo0, bnx;
  double* first;            // first-pass fault states, 22 x nfirst, faces [vlo0-1, vhi0+1]
  double* ffault;           // final fault-face fluxes, 22 x (vhi0-vlo0+1)
  int nfirst;
  Real* Fx;                 // optional reflux fluxes (22 comps over x faces of valid)
  Real* Fy;
  double* Bold;             // fault data at the start of the step (coarse-fine time interpolation)
  double* cap;              // captured face fluxes of the level (flux registers), 22 per slot
  const int4* caplist;      // (dir, i, j, slot) of the captured faces, grouped by tile
  const double* fric;       // optional per-face rate-and-state a, b, L: 3 planes like B (stride bnx)
  const void* tmap;         // TMA tensor map of Uin (x, y, component) for the tile kernel's staged
                            // load, in global memory; null: the tile kernel loads element by element
  DevStatus* status;        // where the tile kernel reports a staged load that never landed
};

// A tile of the volume kernel; [cap0, cap0+ncap) are the captured faces it owns.
struct TileDev { int patch, x0, y0, nx, ny, cap0 = 0, ncap = 0; };

template <typename Real>
TMK_D size_t fab_idx(const PatchDev<Real>& p, int c, int i, int j) {
  return ((size_t)c * (size_t)p.any + (size_t)(j - p.alo1)) * (size_t)p.anx + (size_t)(i - p.alo0);
}

TMK_D void side_bg(const DevParams& P, int s, double* bg) {
#pragma unroll
  for (int c = 0; c < NSIDE; ++c) bg[c] = P.bg[11 * s + c];
}

template <typename T>
TMK_D void make_sig(const DevParams& P, double dtbydx, T* sig) {
  const double l[9] = {-P.cp, -P.cs, -P.cs, 0.0, 0.0, 0.0, P.cs, P.cs, P.cp};
#pragma unroll
  for (int c = 0; c < 9; ++c) sig[c] = (T)(l[c] * dtbydx);
}

// =============================================================== fault kernel
// Predicted state of one side's 11 components at (i, j0) in y, in arithmetic T
// (lambda, gamma carry only their limited PPM delta: zero characteristic speed).
// `tr` (the tracing coefficients A then B of ppm_predict_prim, mixed form with
// PPM and primitive limiting) selects the branch-free predictor.
template <int D, typename T>
TMK_D void fault_pred(const DevParams& P, const Consts<T>& k, T rv, const T (*w5)[5], const bool* in, const T* sig,
                      const T* tr, T* WM, T* WP) {
  if (tr) ppm_predict_prim<D, T>(k, rv, w5, in, tr, tr + NSIDE, WM, WP);
  else ppm_predict<D, T>(k, rv, w5, in, P.prim_lim != 0, P.char_lim != 0, sig, WM, WP, P.order, P.fourth != 0);
}

template <typename Real, typename T>
TMK_D void fault_ypred_side(const PatchDev<Real>& p, const DevParams& P, const Consts<T>& k, int s, int i,
                            const T* sig, const T* tr, bool lim, double* out11) {
  const int j0 = p.dlo1;
  bool in[5] = {false, false, true, j0 + 1 <= p.dhi1, j0 + 2 <= p.dhi1};
  T w5[NSIDE][5];
  for (int c = 0; c < NSIDE; ++c)
    for (int m = 0; m < 5; ++m) w5[c][m] = in[m] ? (T)p.Uin[fab_idx(p, 11 * s + c, i, j0 - 2 + m)] : T(0);
  T WM[NSIDE], WP[NSIDE];
  T rv = (s == 1) ? T(-1) : T(1);
  fault_pred<1, T>(P, k, rv, w5, in, sig, tr, WM, WP);
  // the zero-speed components of the y direction reach no face component that
  // is read downstream (live9): not predicted
  for (int c = 0; c < NSIDE; ++c) out11[c] = live9<1>(c) ? (double)WM[c] : 0.0;
  for (int c = 9; c < 11; ++c) {
    T w[5];
    for (int m = 0; m < 5; ++m) w[m] = in[m] ? (T)p.Uin[fab_idx(p, 11 * s + c, i, j0 - 2 + m)] : T(0);
    if (P.order == 0) { out11[c] = (double)w[2]; continue; }
    if (P.order == 1) {          // PLM: lo-face value of a zero-speed component
      T sl = plm_slope(w, in, lim, P.fourth != 0);
      if (lim && (P.char_lim || P.fourth)) {
        T m, p1;
        plm_onesided(w, in, m, p1);
        sl = plm_limit(sl, m, p1);
      }
      out11[c] = (double)(-T(0.5) * sl + w[2]);
      continue;
    }
    T dm, dp;
    ppm_deltas(w, in, lim, dm, dp);
    if (lim) ppm_limit(dm, dp);
    out11[c] = (double)(dm + w[2]);
  }
}

// x-direction predicted states (WM, WP) of one side at cell (i, j0)
template <typename Real, typename T>
TMK_D void fault_xpred_side(const PatchDev<Real>& p, const DevParams& P, const Consts<T>& k, int s, int i,
                            const T* sig, const T* tr, T* WM, T* WP) {
  const int j0 = p.dlo1;
  bool in[5];
  for (int m = 0; m < 5; ++m) in[m] = (i - 2 + m >= p.dlo0) && (i - 2 + m <= p.dhi0);
  T w5[NSIDE][5];
  for (int c = 0; c < NSIDE; ++c)
    for (int m = 0; m < 5; ++m) w5[c][m] = in[m] ? (T)p.Uin[fab_idx(p, 11 * s + c, i - 2 + m, j0)] : T(0);
  fault_pred<0, T>(P, k, T(1), w5, in, sig, tr, WM, WP);
}

// x face state (first pass) of one side at face f of row j0 from the cells
// f-1 and f, or the domain-edge condition.
template <typename T>
TMK_D void xface_state(const DevParams& P, const Consts<T>& k, int f, int dlo0, int dhi0, const T* WPl,
                       const T* WMr, const T* bg, T* g) {
  if (f == dlo0) edge_bc<0, T>(k, T(1), -1, P.bc[0] == 0, bg, WMr, g);
  else if (f == dhi0 + 1) edge_bc<0, T>(k, T(1), +1, P.bc[1] == 0, bg, WPl, g);
  else riemann<0, T>(k, T(1), WPl, WMr, g);
}

// One CTA of NT threads per segment of SEG fault faces of a fault patch.  The
// predictors of the fault row are computed once per cell and side, in
// parallel, into shared memory; one thread per face then runs the friction
// solves, whose Newton iterations are sequential by nature.  Two variants:
// 32 faces on 4 warps (the default) and 16 faces on 2 warps (twice the CTAs
// for short fault rows); the level's tuning picks one.
constexpr int FAULT_SEG = 32;
constexpr int FAULT_THREADS = 128;
constexpr int FAULT_SEG_SMALL = 16;
constexpr int FAULT_THREADS_SMALL = 64;

template <typename Real, int SEG, int NT>
__global__ void __launch_bounds__(NT) fault_kernel(const PatchDev<Real>* __restrict__ patches,
                                                   const int* __restrict__ fault_patches,
                                                   const DevParams* __restrict__ params, double time,
                                                   DevStatus* st) {
  static_assert(NT > SEG + 2, "the x-face threads need the threads beyond the face threads");
  using T = Real;
  // the mixed form runs the latency-arranged rate-and-state path (per-face
  // constants, z = asinh(beta V) Newton solve); the FP64 form keeps the
  // reference's operation order and Newton iteration on V
  constexpr bool kZSolve = !std::is_same<Real, double>::value;
  constexpr int NCELL = SEG + 2;             // cells / faces [s0-1, s0+SEG]
  __shared__ T xWM[2][NCELL][NSIDE], xWP[2][NCELL][NSIDE];
  __shared__ T H1x[2][SEG + 1][NSIDE];
  __shared__ double sWi[NCELL][NC];
  __shared__ double sTmp[NCELL];
  __shared__ RSFaceK sFk[kZSolve ? NCELL : 1];   // mixed form: per-face rate-and-state constants
  // the kernel launched after this one may be scheduled now (it reads none of
  // this kernel's outputs before it waits for it).  When this kernel itself is
  // a programmatic dependent of the in-plane marching kernel, it reads nothing
  // that kernel writes (the state it reads is the step's input buffer) and it
  // waits for it before exiting, so that the step's kernels complete in order.
  asm volatile("griddepcontrol.launch_dependents;");
  const PatchDev<Real> p = patches[fault_patches[blockIdx.y]];
  const DevParams& P = params[p.scen];
  const int s0 = p.vlo0 + blockIdx.x * SEG;
  if (s0 > p.vhi0) {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    return;
  }
  const int s1 = min(s0 + SEG - 1, p.vhi0);
  // faces whose first-pass state this segment produces: its own, plus the
  // ghost faces lo-1 / hi+1 of the patch for the first / last segment
  const int fa = (s0 == p.vlo0) ? max(p.vlo0 - 1, p.dlo0) : s0;
  const int fb = (s1 == p.vhi0) ? min(p.vhi0 + 1, p.dhi0) : s1;
  const int tid = threadIdx.x;
  const double dt = p.dt, dx = p.dx;
  // the constants once per CTA: computed per thread they were hundreds of FP64
  // divisions and products queued on GB300's narrow FP64 pipe before any face
  // could start
  __shared__ Consts<T> sk;
  __shared__ Consts<double> skd;
  __shared__ T ssig[9];
  __shared__ T str[2 * NSIDE];     // tracing coefficients of the branch-free predictor
  const bool fastpred = !kExact<T> && P.order == 2 && P.prim_lim && !P.char_lim;
  if (tid == 0) {
    sk.load(P);
    skd.load(P);
    make_sig(P, dt / dx, ssig);
    if (fastpred)
      for (int q = 0; q < NSIDE; ++q) {
        const double sv = fabs((double)ssig[q]);
        str[q] = (T)(0.5 * sv);
        str[NSIDE + q] = (T)(q < 3 ? 3.0 * (0.5 * sv - sv * sv / 3.0) : 1.5 * sv * (1.0 - (2.0 / 3.0) * sv));
      }
  }
  __syncthreads();
  const Consts<T>& k = sk;
  const T* sig = ssig;
  const T* tr = fastpred ? str : nullptr;
  const bool lim = P.prim_lim || P.char_lim;
  const int bs = p.bnx;

  // (A) x predictors of the fault-row cells [s0-1, s1+1] and y predictors of the
  //     states entering the fault faces [fa, fb], both sides; in the mixed form
  //     also the constants of each face
  if constexpr (kZSolve) {
    if (P.fault_law == 1 && tid >= NT - NCELL) {
      const int ci = tid - (NT - NCELL), i = s0 - 1 + ci;
      if (i >= fa && i <= fb) sFk[ci] = rs_face_k(P, rs_face(P, p.fric, i - p.blo0, bs), (i + 0.5) * dx - P.rs_x0);
    }
  }
  for (int t = tid; t < 4 * NCELL; t += NT) {
    const int kind = t / (2 * NCELL), s = (t / NCELL) & 1, ci = t % NCELL;
    const int c = s0 - 1 + ci;
    if (kind == 0) {
      if (c >= p.dlo0 && c <= p.dhi0 && c <= s1 + 1) {
        T WM[NSIDE], WP[NSIDE];
        fault_xpred_side(p, P, k, s, c, sig, tr, WM, WP);
        // the x faces' zero-speed components are never read (live9): not predicted
        for (int q = 0; q < NSIDE; ++q) {
          xWM[s][ci][q] = live9<0>(q) ? WM[q] : T(0);
          xWP[s][ci][q] = live9<0>(q) ? WP[q] : T(0);
        }
      }
    } else if (c >= fa && c <= fb) {
      fault_ypred_side(p, P, k, s, c, sig, tr, lim, &sWi[ci][11 * s]);
    }
  }
  __syncthreads();

  if (tid < NCELL) {
    // (B) first-pass friction solve with the persistent boundary data, and the
    //     half-step predicted boundary data (updateBoundary, final=false)
    const int i = s0 - 1 + tid;
    if (i >= fa && i <= fb) {
      double* Bi = p.B + (i - p.blo0);
      const double xc = (i + 0.5) * dx;
      double Wg[NC];
      for (int c = 0; c < NC; ++c) Wg[c] = 0.0;
      int it = 0;
      const RSFace fr = rs_face(P, p.fric, i - p.blo0, bs);
      if (P.fault_law == 1) {
        if constexpr (kZSolve) it = rs_fault_k_ool(P, sFk[tid], sWi[tid], Bi[10 * bs], Wg);
        else it = rs_fault(P, fr, sWi[tid], Bi[10 * bs], xc - P.rs_x0, Wg);
      } else {
        sw_fault(P, sWi[tid], Bi[7 * bs], xc, Wg);
      }
      if (it > RS_IMAX) atomicAdd(&st->newton_maxed, 1ull);
      double* first = p.first + (i - (p.vlo0 - 1));
      for (int c = 0; c < NC; ++c) first[c * p.nfirst] = Wg[c];
      if (i >= s0 && i <= s1) {
        if (P.fault_law == 1) {
          if constexpr (kZSolve) sTmp[tid] = rs_setbnd_k_ool(P, sFk[tid], Wg, Bi, bs, 0.5 * dt, 0.0, false);
          else sTmp[tid] = rs_setbnd(P, fr, Wg, Bi, bs, 0.5 * dt, xc - P.rs_x0, 0.0, false);
        } else {
          sTmp[tid] = sw_setbnd(P, Wg, Bi, bs, 0.5 * dt, 0.0, false);
        }
      }
    }
  } else {
    // (C) first-pass x faces [s0, s1+1] of the fault row, both sides
    for (int t = tid - NCELL; t < 2 * (SEG + 1); t += NT - NCELL) {
      const int s = t / (SEG + 1), fi = t % (SEG + 1);
      const int f = s0 + fi;
      if (f > s1 + 1) continue;
      double bgd[NSIDE]; side_bg(P, s, bgd);
      T bg[NSIDE];
      for (int c = 0; c < NSIDE; ++c) bg[c] = (T)bgd[c];
      T g[NSIDE];
      xface_state<T>(P, k, f, p.dlo0, p.dhi0, xWP[s][fi], xWM[s][fi + 1], bg, g);
      for (int q = 0; q < NSIDE; ++q) H1x[s][fi][q] = g[q];
    }
  }
  __syncthreads();

  if (tid <= s1 - s0) {
    const int i = s0 + tid, ci = tid + 1;
    double* Bi = p.B + (i - p.blo0);
    const double xc = (i + 0.5) * dx;
    // (D) transverse correction of the fault states by the x fluxes of the row
    const double scale = -(1.0 / 2.0) * dt / dx;
    double Wi[NC];
    for (int c = 0; c < NC; ++c) Wi[c] = sWi[ci][c];
    for (int s = 0; s < 2; ++s) {
      T q[NSIDE];
      for (int c = 0; c < NSIDE; ++c) q[c] = (T)Wi[11 * s + c];
      adwdx_add<0, T>(k, T(1), (T)scale, H1x[s][tid + 1], H1x[s][tid], q);
      for (int c = 0; c < NSIDE; ++c) Wi[11 * s + c] = (double)q[c];
    }
    // (E) final friction solve with the predicted boundary data
    double Wg[NC];
    for (int c = 0; c < NC; ++c) Wg[c] = 0.0;
    int it = 0;
    const RSFace fr = rs_face(P, p.fric, i - p.blo0, bs);
    if (P.fault_law == 1) {
      if constexpr (kZSolve) it = rs_fault_k_ool(P, sFk[ci], Wi, sTmp[ci], Wg);
      else it = rs_fault(P, fr, Wi, sTmp[ci], xc - P.rs_x0, Wg);
    } else {
      sw_fault(P, Wi, sTmp[ci], xc, Wg);
    }
    if (it > RS_IMAX) atomicAdd(&st->newton_maxed, 1ull);
    // (F) y fluxes through the fault face (GETFLUXF, FP64)
    const Consts<double>& kd = skd;
    double F[NSIDE];
    double* ff = p.ffault + (i - p.vlo0);
    const int nv = p.vhi0 - p.vlo0 + 1;
    flux<1, double>(kd, 1.0, Wg, F);
    for (int c = 0; c < NSIDE; ++c) ff[c * nv] = F[c];
    flux<1, double>(kd, -1.0, Wg + 11, F);
    for (int c = 0; c < NSIDE; ++c) ff[(11 + c) * nv] = F[c];
    // (G) boundary-data update with the final fault state (final=true, t+dt)
    if (P.fault_law == 1) {
      double np;
      if constexpr (kZSolve) np = rs_setbnd_k_ool(P, sFk[ci], Wg, Bi, bs, dt, time + dt, true);
      else np = rs_setbnd(P, fr, Wg, Bi, bs, dt, xc - P.rs_x0, time + dt, true);
      if (isnan(np)) report(st, ST_NAN, (long long)i);
    } else {
      sw_setbnd(P, Wg, Bi, bs, dt, time + dt, true);
    }
  }
  asm volatile("griddepcontrol.wait;" ::: "memory");
}

// ============================================================== volume kernel
template <typename Real, int TX, int TY>
struct VolSmem {
  static constexpr int RX = TX + 6, RY = TY + 6, PX = TX + 2, PY = TY + 2;
  // staged rows: RXP columns from the 16-byte boundary at or before the
  // tile's first halo column (a TMA box starts on a 16-byte boundary in x)
  static constexpr int AX = 16 / (int)sizeof(Real);
  static constexpr int RXP = (RX + AX - 1 + AX - 1) / AX * AX;
  Real W[NSIDE][RY][RXP];
  Real WMx[NSIDE][PY][PX], WPx[NSIDE][PY][PX];
  Real WMy[NSIDE][PY][PX], WPy[NSIDE][PY][PX];
  Real H1x[NSIDE][PY][TX + 1];
  Real H1y[NSIDE][TY + 1][PX];
  Real Fx[NSIDE][TY][TX + 1];
  Real Fy[NSIDE][TY + 1][TX];
  unsigned long long bar;        // mbarrier of the staged load
};

// ---- TMA: one tensor copy of a box (x, y, component) into shared memory,
// completion counted on an mbarrier
TMK_D unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
TMK_D void mbar_init(unsigned long long* bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)) : "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");   // visible to the copy engine
}
TMK_D void tma_load_3d(void* dst, const void* tmap, int x, int y, int z, unsigned long long* bar, unsigned bytes) {
  // the map sits in global memory, written by a copy from the host: order it for the tensormap proxy
  asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(tmap) : "memory");
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
      ::"r"(smem_u32(dst)), "l"(tmap), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar)) : "memory");
}
// Wait for phase `parity` of the mbarrier, at most `limit` polls; false if it never completed.
TMK_D bool mbar_wait(unsigned long long* bar, unsigned parity, int limit) {
  for (int i = 0; i < limit; ++i) {
    unsigned done;
    asm volatile("{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
                 : "=r"(done) : "r"(smem_u32(bar)), "r"(parity) : "memory");
    if (done) return true;
  }
  return false;
}
constexpr int TMA_WAIT_POLLS = 1 << 20;

template <typename Real, int TX, int TY, int NT>
__global__ void __launch_bounds__(NT) volume_kernel(const PatchDev<Real>* __restrict__ patches,
                                                    const TileDev* __restrict__ tiles,
                                                    const DevParams* __restrict__ params) {
  using T = Real;
  using S = VolSmem<Real, TX, TY>;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  S& sm = *reinterpret_cast<S*>(smem_raw);
  const TileDev tl = tiles[blockIdx.x];
  const int s = blockIdx.y;                // side
  const PatchDev<Real>& pp = patches[tl.patch];
  const PatchDev<Real> p = pp;
  const DevParams& P = params[p.scen];
  Consts<T> k; k.load(P);
  const T rvy = (s == 1) ? T(-1) : T(1);
  const int x0 = tl.x0, y0 = tl.y0, tnx = tl.nx, tny = tl.ny;
  const double dt = p.dt, dx = p.dx;
  const bool plim = P.prim_lim != 0, clim = P.char_lim != 0;
  T sig[9]; make_sig(P, dt / dx, sig);
  const T scale = (T)(-(1.0 / 2.0) * dt / dx);
  const T sc = (T)(-dt / dx);
  double bgd[NSIDE]; side_bg(P, s, bgd);
  T bg[NSIDE];
  for (int c = 0; c < NSIDE; ++c) bg[c] = (T)bgd[c];
  const bool outx_lo = P.bc[0] == 0, outx_hi = P.bc[1] == 0;
  const bool outy_lo = P.bc[2] == 0, outy_hi = P.bc[3] == 0;

  // ---- stage W over [x0-3, x0+TX+2] x [y0-3, y0+TY+2]; column x0-3+q sits at W[..][q + wo]
  int wo = 0;
  if (p.tmap) {
    // one TMA tensor copy of the side's 11 components over the tile and its halo,
    // from the 16-byte boundary at or before x0-3 (cells beyond the FAB read 0)
    const int xr = x0 - 3 - p.alo0;
    wo = ((xr % S::AX) + S::AX) % S::AX;
    if (threadIdx.x == 0) mbar_init(&sm.bar);
    __syncthreads();
    if (threadIdx.x == 0)
      tma_load_3d(&sm.W[0][0][0], p.tmap, xr - wo, y0 - 3 - p.alo1, 11 * s, &sm.bar,
                  (unsigned)(NSIDE * S::RY * S::RXP * sizeof(Real)));
    const bool landed = mbar_wait(&sm.bar, 0, TMA_WAIT_POLLS);
    if (__syncthreads_or(!landed)) {     // the whole CTA agrees
      // the copy never landed: record it, give it one more bounded wait, leave
      if (threadIdx.x == 0 && p.status) report(p.status, ST_TIMEOUT, (long long)blockIdx.x);
      mbar_wait(&sm.bar, 0, TMA_WAIT_POLLS);
      return;
    }
    // cells outside the domain stage as zeros, as the element-wise load leaves them
    if (x0 - 3 < p.dlo0 || x0 + tnx + 2 > p.dhi0 || y0 - 3 < p.dlo1 || y0 + tny + 2 > p.dhi1) {
      for (int idx = threadIdx.x; idx < NSIDE * S::RY * S::RX; idx += NT) {
        int c = idx / (S::RY * S::RX), r = (idx / S::RX) % S::RY, q = idx % S::RX;
        int x = x0 - 3 + q, y = y0 - 3 + r;
        if (x < p.dlo0 || x > p.dhi0 || y < p.dlo1 || y > p.dhi1) sm.W[c][r][q + wo] = T(0);
      }
      __syncthreads();
    }
  } else {
    for (int idx = threadIdx.x; idx < NSIDE * S::RY * S::RX; idx += NT) {
      int c = idx / (S::RY * S::RX), r = (idx / S::RX) % S::RY, q = idx % S::RX;
      int x = x0 - 3 + q, y = y0 - 3 + r;
      T v = T(0);
      if (x >= p.dlo0 && x <= p.dhi0 && y >= p.dlo1 && y <= p.dhi1 && q < tnx + 6 && r < tny + 6)
        v = p.Uin[fab_idx(p, 11 * s + c, x, y)];
      sm.W[c][r][q] = v;
    }
    __syncthreads();
  }

  // ---- normal predictors on cells [x0-1, x0+nx] x [y0-1, y0+ny]
  for (int idx = threadIdx.x; idx < (tny + 2) * (tnx + 2); idx += NT) {
    int py = idx / (tnx + 2), px = idx % (tnx + 2);
    int x = x0 - 1 + px, y = y0 - 1 + py;
    if (x < p.dlo0 || x > p.dhi0 || y < p.dlo1 || y > p.dhi1) continue;
    T w5[NSIDE][5], WM[NSIDE], WP[NSIDE];
    bool in[5];
#pragma unroll
    for (int m = 0; m < 5; ++m) in[m] = (x - 2 + m >= p.dlo0) && (x - 2 + m <= p.dhi0);
#pragma unroll
    for (int c = 0; c < NSIDE; ++c)
#pragma unroll
      for (int m = 0; m < 5; ++m) w5[c][m] = sm.W[c][py + 2][px + m + wo];
    ppm_predict<0, T>(k, T(1), w5, in, plim, clim, sig, WM, WP, P.order, P.fourth != 0);
#pragma unroll
    for (int c = 0; c < NSIDE; ++c) { sm.WMx[c][py][px] = WM[c]; sm.WPx[c][py][px] = WP[c]; }
#pragma unroll
    for (int m = 0; m < 5; ++m) in[m] = (y - 2 + m >= p.dlo1) && (y - 2 + m <= p.dhi1);
#pragma unroll
    for (int c = 0; c < NSIDE; ++c)
#pragma unroll
      for (int m = 0; m < 5; ++m) w5[c][m] = sm.W[c][py + m][px + 2 + wo];
    ppm_predict<1, T>(k, rvy, w5, in, plim, clim, sig, WM, WP, P.order, P.fourth != 0);
#pragma unroll
    for (int c = 0; c < NSIDE; ++c) { sm.WMy[c][py][px] = WM[c]; sm.WPy[c][py][px] = WP[c]; }
  }
  __syncthreads();

  // ---- first-pass Riemann: x faces [x0, x0+nx] on rows [y0-1, y0+ny]
  for (int idx = threadIdx.x; idx < (tny + 2) * (tnx + 1); idx += NT) {
    int ry = idx / (tnx + 1), fi = idx % (tnx + 1);
    int f = x0 + fi, y = y0 - 1 + ry;
    if (y < p.dlo1 || y > p.dhi1) continue;
    T L[NSIDE], R[NSIDE], g[NSIDE];
#pragma unroll
    for (int c = 0; c < NSIDE; ++c) { L[c] = sm.WPx[c][ry][fi]; R[c] = sm.WMx[c][ry][fi + 1]; }
    if (f == p.dlo0) edge_bc<0, T>(k, T(1), -1, outx_lo, bg, R, g);
    else if (f == p.dhi0 + 1) edge_bc<0, T>(k, T(1), +1, outx_hi, bg, L, g);
    else riemann<0, T>(k, T(1), L, R, g);
#pragma unroll
    for (int c = 0; c < NSIDE; ++c) sm.H1x[c][ry][fi] = g[c];
  }
  //      y faces [y0, y0+ny] on columns [x0-1, x0+nx]
  for (int idx = threadIdx.x; idx < (tny + 1) * (tnx + 2); idx += NT) {
    int gi = idx / (tnx + 2), cx = idx % (tnx + 2);
    int gf = y0 + gi, x = x0 - 1 + cx;
    if (x < p.dlo0 || x > p.dhi0) continue;
    T g[NSIDE];
    if (gf == p.dlo1 && p.fault) {
      const double* fs = p.first + (x - (p.vlo0 - 1)) + (size_t)(11 * s) * p.nfirst;
#pragma unroll
      for (int c = 0; c < NSIDE; ++c) g[c] = (T)fs[c * p.nfirst];
    } else {
      T L[NSIDE], R[NSIDE];
#pragma unroll
      for (int c = 0; c < NSIDE; ++c) { L[c] = sm.WPy[c][gi][cx]; R[c] = sm.WMy[c][gi + 1][cx]; }
      if (gf == p.dlo1) edge_bc<1, T>(k, rvy, -1, outy_lo, bg, R, g);
      else if (gf == p.dhi1 + 1) edge_bc<1, T>(k, rvy, +1, outy_hi, bg, L, g);
      else riemann<1, T>(k, rvy, L, R, g);
    }
#pragma unroll
    for (int c = 0; c < NSIDE; ++c) sm.H1y[c][gi][cx] = g[c];
  }
  __syncthreads();

  // ---- transverse corrections (quasilinearUpdate with -(1/2) dt/dx)
  for (int idx = threadIdx.x; idx < tny * (tnx + 2); idx += NT) {
    int ry = idx / (tnx + 2), px = idx % (tnx + 2);
    int x = x0 - 1 + px;
    if (x < p.dlo0 || x > p.dhi0) continue;
    T h[NSIDE], l[NSIDE], a[NSIDE];
#pragma unroll
    for (int c = 0; c < NSIDE; ++c) { h[c] = sm.H1y[c][ry + 1][px]; l[c] = sm.H1y[c][ry][px]; a[c] = T(0); }
    adwdx_add<1, T>(k, rvy, scale, h, l, a);
#pragma unroll
    for (int c = 0; c < NSIDE; ++c) { sm.WMx[c][ry + 1][px] += a[c]; sm.WPx[c][ry + 1][px] += a[c]; }
  }
  for (int idx = threadIdx.x; idx < (tny + 2) * tnx; idx += NT) {
    int py = idx / tnx, cx = idx % tnx;
    int y = y0 - 1 + py;
    if (y < p.dlo1 || y > p.dhi1) continue;
    T h[NSIDE], l[NSIDE], a[NSIDE];
#pragma unroll
    for (int c = 0; c < NSIDE; ++c) { h[c] = sm.H1x[c][py][cx + 1]; l[c] = sm.H1x[c][py][cx]; a[c] = T(0); }
    adwdx_add<0, T>(k, T(1), scale, h, l, a);
#pragma unroll
    for (int c = 0; c < NSIDE; ++c) { sm.WMy[c][py][cx + 1] += a[c]; sm.WPy[c][py][cx + 1] += a[c]; }
  }
  __syncthreads();

  // ---- final Riemann + fluxes: x faces [x0, x0+nx] on rows [y0, y0+ny-1]
  for (int idx = threadIdx.x; idx < tny * (tnx + 1); idx += NT) {
    int ry = idx / (tnx + 1), fi = idx % (tnx + 1);
    int f = x0 + fi;
    T L[NSIDE], R[NSIDE], g[NSIDE], F[NSIDE];
#pragma unroll
    for (int c = 0; c < NSIDE; ++c) { L[c] = sm.WPx[c][ry + 1][fi]; R[c] = sm.WMx[c][ry + 1][fi + 1]; }
    if (f == p.dlo0) edge_bc<0, T>(k, T(1), -1, outx_lo, bg, R, g);
    else if (f == p.dhi0 + 1) edge_bc<0, T>(k, T(1), +1, outx_hi, bg, L, g);
    else riemann<0, T>(k, T(1), L, R, g);
    flux<0, T>(k, T(1), g, F);
#pragma unroll
    for (int c = 0; c < NSIDE; ++c) sm.Fx[c][ry][fi] = F[c];
  }
  //      y faces [y0, y0+ny] on columns [x0, x0+nx-1]
  for (int idx = threadIdx.x; idx < (tny + 1) * tnx; idx += NT) {
    int gi = idx / tnx, cx = idx % tnx;
    int gf = y0 + gi, x = x0 + cx;
    T F[NSIDE];
    if (gf == p.dlo1 && p.fault) {
      const int nv = p.vhi0 - p.vlo0 + 1;
      const double* ff = p.ffault + (x - p.vlo0) + (size_t)(11 * s) * nv;
#pragma unroll
      for (int c = 0; c < NSIDE; ++c) F[c] = (T)ff[c * nv];
    } else {
      T L[NSIDE], R[NSIDE], g[NSIDE];
#pragma unroll
      for (int c = 0; c < NSIDE; ++c) { L[c] = sm.WPy[c][gi][cx + 1]; R[c] = sm.WMy[c][gi + 1][cx + 1]; }
      if (gf == p.dlo1) edge_bc<1, T>(k, rvy, -1, outy_lo, bg, R, g);
      else if (gf == p.dhi1 + 1) edge_bc<1, T>(k, rvy, +1, outy_hi, bg, L, g);
      else riemann<1, T>(k, rvy, L, R, g);
      flux<1, T>(k, rvy, g, F);
    }
#pragma unroll
    for (int c = 0; c < NSIDE; ++c) sm.Fy[c][gi][cx] = F[c];
  }
  __syncthreads();

  // ---- conservative update (LinElastPhysics::computeUpdate) + plasticity
  for (int idx = threadIdx.x; idx < tny * tnx; idx += NT) {
    int ry = idx / tnx, cx = idx % tnx;
    int x = x0 + cx, y = y0 + ry;
    T u[NSIDE];
#pragma unroll
    for (int c = 0; c < NSIDE; ++c) {
      T du = (sm.Fx[c][ry][cx + 1] - sm.Fx[c][ry][cx]) + (sm.Fy[c][ry + 1][cx] - sm.Fy[c][ry][cx]);
      u[c] = sm.W[c][ry + 3][cx + 3 + wo] + du * sc;
    }
    if (p.plastic) {
      T lam = p.Uin[fab_idx(p, 11 * s + 9, x, y)];
      T gam = p.Uin[fab_idx(p, 11 * s + 10, x, y)];
      plastic_flow<T>(P, u[3], u[4], u[5], u[6], u[7], u[8], lam, gam, (T)dt);
      p.Uout[fab_idx(p, 11 * s + 9, x, y)] = lam;
      p.Uout[fab_idx(p, 11 * s + 10, x, y)] = gam;
    }
#pragma unroll
    for (int c = 0; c < NSIDE; ++c) p.Uout[fab_idx(p, 11 * s + c, x, y)] = u[c];
  }
  if (p.Fx) {
    const int nvx = p.vhi0 - p.vlo0 + 2, nvy = p.vhi1 - p.vlo1 + 1;
    for (int idx = threadIdx.x; idx < NSIDE * tny * (tnx + 1); idx += NT) {
      int c = idx / (tny * (tnx + 1)), ry = (idx / (tnx + 1)) % tny, fi = idx % (tnx + 1);
      size_t o = ((size_t)(11 * s + c) * nvy + (y0 + ry - p.vlo1)) * nvx + (x0 + fi - p.vlo0);
      p.Fx[o] = sm.Fx[c][ry][fi];
    }
  }
  if (p.Fy) {
    const int nvx = p.vhi0 - p.vlo0 + 1, nvy = p.vhi1 - p.vlo1 + 2;
    for (int idx = threadIdx.x; idx < NSIDE * (tny + 1) * tnx; idx += NT) {
      int c = idx / ((tny + 1) * tnx), gi = (idx / tnx) % (tny + 1), cx = idx % tnx;
      size_t o = ((size_t)(11 * s + c) * nvy + (y0 + gi - p.vlo1)) * nvx + (x0 + cx - p.vlo0);
      p.Fy[o] = sm.Fy[c][gi][cx];
    }
  }
  // flux-register faces owned by this tile (LevelFluxRegister increments)
  for (int q = threadIdx.x; q < tl.ncap * NSIDE; q += NT) {
    const int4 cr = p.caplist[tl.cap0 + q / NSIDE];
    const int c = q % NSIDE;
    const T v = cr.x == 0 ? sm.Fx[c][cr.z - y0][cr.y - x0] : sm.Fy[c][cr.z - y0][cr.y - x0];
    p.cap[(size_t)cr.w * 22 + 11 * s + c] = (double)v;
  }
}

// =============================================================== plasticity
// PLASTICCORRECTION (srcLinElast/PlasticPhysicsF.ChF:30-69) over the valid
// cells of a level after the marching kernels wrote the updated stresses:
// one thread per cell of a tile, both sides.  lambda and gamma are read from
// the step's input buffer (the volume update leaves them unchanged) and both
// are written to the output buffer.
template <typename Real>
__global__ void __launch_bounds__(256) plastic_tiles_kernel(const PatchDev<Real>* __restrict__ patches,
                                                            const TileDev* __restrict__ tiles,
                                                            const DevParams* __restrict__ params) {
  using T = Real;
  const TileDev tl = tiles[blockIdx.x];
  const PatchDev<Real>& p = patches[tl.patch];
  // the parameters in T once per CTA (FP64-to-FP32 conversions use GB300's
  // narrow FP64 pipe: per cell they were the pass's bound)
  __shared__ PlasticK<T> sk;
  __shared__ T sdt;
  if (threadIdx.x == 0) {
    sk.load(params[p.scen]);
    sdt = (T)p.dt;
  }
  __syncthreads();
  const T dt = sdt;
  for (int idx = threadIdx.x; idx < tl.nx * tl.ny; idx += blockDim.x) {
    const int x = tl.x0 + idx % tl.nx, y = tl.y0 + idx / tl.nx;
    const size_t o = fab_idx(p, 0, x, y), plane = (size_t)p.anx * p.any;
    // both sides' stresses and hardening first: the stores below may alias
    // them for the compiler, which would otherwise wait for one side's stores
    // before loading the other's
    T u[2][6], gam[2];
#pragma unroll
    for (int s = 0; s < 2; ++s) {
#pragma unroll
      for (int c = 0; c < 6; ++c) u[s][c] = p.Uout[o + (size_t)(11 * s + 3 + c) * plane];
      gam[s] = p.Uin[o + (size_t)(11 * s + 10) * plane];
    }
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      T lam;                                   // the plastic rate is only written
      // the stresses are stored back only where the point yielded (else unchanged)
      if (plastic_flow_k<T>(sk, u[s][0], u[s][1], u[s][2], u[s][3], u[s][4], u[s][5], lam, gam[s], dt)) {
#pragma unroll
        for (int c = 0; c < 6; ++c) p.Uout[o + (size_t)(11 * s + 3 + c) * plane] = u[s][c];
      }
      p.Uout[o + (size_t)(11 * s + 9) * plane] = lam;
      p.Uout[o + (size_t)(11 * s + 10) * plane] = gam[s];
    }
  }
}

// =============================================================== exchange
// Copy `ncomp` planes (first component c0) of box [lo, hi] from src to dst.
struct CopyDev { int src, dst; int lo0, lo1, hi0, hi1; };

template <typename Real>
__global__ void exchange_kernel(const PatchDev<Real>* __restrict__ patches, const CopyDev* __restrict__ copies,
                                int c0, int ncomp, int to_in) {
  const CopyDev cp = copies[blockIdx.x];
  const PatchDev<Real>& ps = patches[cp.src];
  const PatchDev<Real>& pd = patches[cp.dst];
  const int nx = cp.hi0 - cp.lo0 + 1, ny = cp.hi1 - cp.lo1 + 1;
  const Real* src = (to_in ? ps.Uout : ps.Uin) + fab_idx(ps, c0, cp.lo0, cp.lo1);
  Real* dst = (to_in ? (Real*)pd.Uout : (Real*)pd.Uin) + fab_idx(pd, c0, cp.lo0, cp.lo1);
  const size_t splane = (size_t)ps.any * ps.anx, dplane = (size_t)pd.any * pd.anx;
  const int nrow = ncomp * ny;
  const int step = blockDim.x * gridDim.y, t0 = threadIdx.x + blockIdx.y * blockDim.x;
  // rows of 16-byte vectors when every row of both boxes starts on a 16-byte boundary
  constexpr int W = 16 / sizeof(Real);
  const bool vec = nx % W == 0 && ps.anx % W == 0 && pd.anx % W == 0 && splane % W == 0 && dplane % W == 0 &&
                   ((uintptr_t)src & 15) == 0 && ((uintptr_t)dst & 15) == 0;
  if (vec) {
    // four vectors per thread in flight: all loads, then all stores
    constexpr int U = 4;
    const int nv = nx / W, n = nrow * nv;
    for (int base = t0; base < n; base += U * step) {
      float4 v[U];
      size_t o[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int idx = base + u * step;
        if (idx < n) {
          const int row = idx / nv, k = idx - row * nv, c = row / ny, j = row - c * ny;
          v[u] = __ldg((const float4*)(src + c * splane + (size_t)j * ps.anx + k * W));
          o[u] = c * dplane + (size_t)j * pd.anx + k * W;
        }
      }
#pragma unroll
      for (int u = 0; u < U; ++u)
        if (base + u * step < n) *(float4*)(dst + o[u]) = v[u];
    }
    return;
  }
  // a copy box is spread over gridDim.y CTAs (more loads in flight)
  for (int idx = t0; idx < nrow * nx; idx += step) {
    const int row = idx / nx, i = idx - row * nx, c = row / ny, j = row - c * ny;
    dst[c * dplane + (size_t)j * pd.anx + i] = src[c * splane + (size_t)j * ps.anx + i];
  }
}

}  // namespace tmk
