// The 3-D patch step (CH_SPACEDIM == 3): the C ABI and the plain FP64 form.
// Compiled with --fmad=false so that every product and sum of the FP64 form
// rounds as in the reference's Fortran and the CPU oracle.  The kernels are in
// tmk_3d.cuh; the mixed form's instantiation is in tmk_3d_f32.cu.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "tmk_internal.h"
#include "tmk_3d.cuh"

namespace tmk {
namespace d3 {

cudaError_t launch_step_f64(const Step3<double>& g, const DevParams* P, DevStatus* st, cudaStream_t s,
                            const Side* side) {
  return launch_step<double>(g, P, st, s, side);
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

// make_sig on the host (the same FP64 products, rounded to T)
template <typename T>
void make_sig_host(const tmk::DevParams& P, double dtbydx, T* sig) {
  const double l[9] = {-P.cp, -P.cs, -P.cs, 0.0, 0.0, 0.0, P.cs, P.cs, P.cp};
  for (int c = 0; c < 9; ++c) sig[c] = (T)(l[c] * dtbydx);
}

}  // namespace

namespace {

// fill the boxes and scratch pointers of a step in arithmetic T and launch it
template <typename T>
tmk_status step3(tmk_context* c, tmk::d3::Step3<T>& g, cudaStream_t s) {
  using namespace tmk::d3;
  // scratch: WM, WP (3 each) | WH1 (3) | WH2 (6) | WH (3) | LG | FF (3) | FP32 copy of U
  const size_t s18 = (size_t)NF * g.S.cells() * sizeof(T);
  constexpr bool copy = !std::is_same<T, double>::value;
  std::vector<size_t> sizes;
  for (int d = 0; d < 6; ++d) sizes.push_back(s18);
  for (int d = 0; d < 3; ++d) sizes.push_back((size_t)NF * g.fl1[d].cells() * sizeof(T));
  for (int d1 = 0; d1 < 3; ++d1)
    for (int d2 = 0; d2 < 3; ++d2)
      if (d1 != d2) sizes.push_back((size_t)NF * g.fl1[d1].cells() * sizeof(T));
  for (int d = 0; d < 3; ++d) sizes.push_back((size_t)NF * g.flF[d].cells() * sizeof(T));
  sizes.push_back(2 * (size_t)g.fplane.cells() * sizeof(double));
  for (int k = 0; k < 3; ++k) sizes.push_back((size_t)TMK_NCOMP * g.fplane.cells() * sizeof(double));
  sizes.push_back(copy ? (size_t)NS * g.Ap.cells() * sizeof(T) : 0);
  size_t total = 0;
  for (size_t z : sizes) total += align_up3(z);
  if (total > c->scratch_bytes) {
    TMK_CU(cudaStreamSynchronize(s));
    cudaFree(c->scratch);
    c->scratch = nullptr; c->scratch_bytes = 0;
    if (cudaMalloc(&c->scratch, total) != cudaSuccess) return TMK_ERR_ALLOC;
    c->scratch_bytes = total;
  }
  char* base = (char*)c->scratch;
  size_t off = 0, n = 0;
  auto take = [&]() { char* p = base + off; off += align_up3(sizes[n++]); return p; };
  for (int d = 0; d < 3; ++d) g.WM[d] = (T*)take();
  for (int d = 0; d < 3; ++d) g.WP[d] = (T*)take();
  for (int d = 0; d < 3; ++d) g.WH1[d] = (T*)take();
  for (int d1 = 0; d1 < 3; ++d1)
    for (int d2 = 0; d2 < 3; ++d2)
      if (d1 != d2) g.WH2[d1][d2] = (T*)take();
  for (int d = 0; d < 3; ++d) g.WH[d] = (T*)take();
  g.LG = (double*)take();
  for (int k = 0; k < 3; ++k) g.FF[k] = (double*)take();
  T* up = (T*)take();
  if constexpr (copy) { g.Up = up; g.Uc = up; g.uside = tmk::NSIDE; }
  else { g.Up = (const T*)(const void*)g.U; g.Uc = nullptr; g.Ap = g.A; g.uside = 11; }
  g.kc.load(c->hp);
  make_sig_host(c->hp, g.dt / g.dx, g.sig);
  g.scale3 = (T)(-(1.0 / 3.0) * g.dt / g.dx);
  g.scale2 = (T)(-(1.0 / 2.0) * g.dt / g.dx);
  g.sc = -g.dt / g.dx;
  g.fastpred = copy && c->hp.order == 2 && c->hp.prim_lim && !c->hp.char_lim;
  for (int q = 0; q < tmk::NSIDE; ++q) {
    const double sv = std::fabs((double)g.sig[q]);
    g.trA[q] = (T)(0.5 * sv);
    g.trB[q] = (T)(q < 3 ? 3.0 * (0.5 * sv - sv * sv / 3.0) : 1.5 * sv * (1.0 - (2.0 / 3.0) * sv));
  }
  // the side stream and events of the overlapped schedule, made once per context
  Side side;
  if (g.fault) {
    if (!c->side) {
      cudaStream_t ss = nullptr;
      if (cudaStreamCreateWithFlags(&ss, cudaStreamNonBlocking) != cudaSuccess) return TMK_ERR_CUDA;
      c->side = ss;
      for (int q = 0; q < 6; ++q)
        if (cudaEventCreateWithFlags(&c->side_ev[q], cudaEventDisableTiming) != cudaSuccess) return TMK_ERR_CUDA;
    }
    side.s = c->side;
    for (int q = 0; q < 6; ++q) side.ev[q] = c->side_ev[q];
  }
  cudaError_t e;
  if constexpr (std::is_same<T, double>::value) e = launch_step_f64(g, c->dp, c->dstatus, s, &side);
  else e = launch_step_f32(g, c->dp, c->dstatus, s, &side);
  return e == cudaSuccess ? TMK_OK : TMK_ERR_CUDA;
}

// validate the descriptors, fill the step's boxes and run it in arithmetic T
template <typename T>
tmk_status patch3(tmk_context* c, const tmk_fab3* U, const tmk_fab3* B, const tmk_fab3* const* Fo,
                  const tmk_box3* valid, const tmk_box3* domain, double dx, double time, double dt,
                  cudaStream_t s) {
  using namespace tmk::d3;
  const Bx cur = bx_of(valid->lo, valid->hi), dom = bx_of(domain->lo, domain->hi), A = bx_of(U->lo, U->hi);
  if (!bx_ok(cur) || !bx_ok(dom) || !bx_ok(A) || !bx_contains(dom, cur)) return TMK_ERR_BAD_DESC;
  if (!bx_contains(A, bx_isect(bx_grow(cur, 3), dom))) return TMK_ERR_BAD_DESC;
  Step3<T> g;
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
  for (int d = 0; d < 3; ++d) {
    if (!Fo[d]) continue;
    if (!Fo[d]->data || Fo[d]->ncomp != TMK_NCOMP) return TMK_ERR_BAD_DESC;
    const Bx fb = bx_of(Fo[d]->lo, Fo[d]->hi);
    for (int e = 0; e < 3; ++e)
      if (fb.lo[e] != g.flF[d].lo[e] || fb.n[e] != g.flF[d].n[e]) return TMK_ERR_BAD_DESC;
    g.F[d] = Fo[d]->data;
  }
  g.U = U->data;
  g.Ap = bx_isect(bx_grow(cur, 3), dom);
  g.dx = dx; g.dt = dt; g.time = time;
  return step3<T>(c, g, s);
}

}  // namespace

extern "C" tmk_status tmk_patch_update_state_3d(tmk_context* c, const tmk_fab3* U, const tmk_fab3* B,
                                                const tmk_fab3* F0, const tmk_fab3* F1, const tmk_fab3* F2,
                                                const tmk_box3* valid, const tmk_box3* domain, double dx,
                                                double time, double dt, double* max_wave_speed, void* stream) {
  if (!c || !U || !U->data || !valid || !domain) return TMK_ERR_BAD_DESC;
  if (U->ncomp != TMK_NCOMP || !(dx > 0) || !(dt > 0)) return TMK_ERR_BAD_DESC;
  const tmk_fab3* Fo[3] = {F0, F1, F2};
  cudaStream_t s = (cudaStream_t)stream;
  // precision follows the scheme: the mixed form keeps U, the friction solves
  // and the boundary data in FP64 and runs the volume stencil in FP32
  const tmk_status r = c->scheme.precision == TMK_PREC_MIXED
                           ? patch3<float>(c, U, B, Fo, valid, domain, dx, time, dt, s)
                           : patch3<double>(c, U, B, Fo, valid, domain, dx, time, dt, s);
  if (r != TMK_OK) return r;
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
