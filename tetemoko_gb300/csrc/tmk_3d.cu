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

cudaError_t launch_one_f64(const PlanOne<double>& pl, const DevParams* P, DevStatus* st, cudaStream_t s,
                           const Side* side) {
  return launch_plan<double>(pl, P, st, s, side);
}
cudaError_t launch_many_f64(const PlanMany<double>& pl, const DevParams* P, DevStatus* st, cudaStream_t s,
                            const Side* side) {
  return launch_plan<double>(pl, P, st, s, side);
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
// a non-empty box whose node box holds fewer than 2^31 points (the kernels
// index the cells of a box, and of its node boxes, in 32 bits)
bool bx_ok(const Bx& b) {
  return b.n[0] > 0 && b.n[1] > 0 && b.n[2] > 0 &&
         (long long)(b.n[0] + 1) * (b.n[1] + 1) * (b.n[2] + 1) < (1LL << 31);
}
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

using tmk::d3::Step3;

// Validate one patch's descriptors and fill its step's boxes, pointers and
// launch constants (scratch pointers are laid out by layout3).
template <typename T>
tmk_status fill3(tmk_context* c, const tmk_fab3* U, const tmk_fab3* B, const tmk_fab3* const* Fo,
                 const tmk_box3* valid, const tmk_box3* domain, double dx, double time, double dt, Step3<T>& g) {
  using namespace tmk::d3;
  if (!U || !U->data || !valid || U->ncomp != TMK_NCOMP) return TMK_ERR_BAD_DESC;
  const Bx cur = bx_of(valid->lo, valid->hi), dom = bx_of(domain->lo, domain->hi), A = bx_of(U->lo, U->hi);
  if (!bx_ok(cur) || !bx_ok(dom) || !bx_ok(A) || !bx_contains(dom, cur)) return TMK_ERR_BAD_DESC;
  if (!bx_contains(A, bx_isect(bx_grow(cur, 3), dom))) return TMK_ERR_BAD_DESC;
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
    if (!Fo || !Fo[d]) continue;
    if (!Fo[d]->data || Fo[d]->ncomp != TMK_NCOMP) return TMK_ERR_BAD_DESC;
    const Bx fb = bx_of(Fo[d]->lo, Fo[d]->hi);
    for (int e = 0; e < 3; ++e)
      if (fb.lo[e] != g.flF[d].lo[e] || fb.n[e] != g.flF[d].n[e]) return TMK_ERR_BAD_DESC;
    g.F[d] = Fo[d]->data;
  }
  g.U = U->data;
  g.Ap = bx_isect(bx_grow(cur, 3), dom);
  g.dx = dx; g.dt = dt; g.time = time;
  // launch constants (the same FP64 expressions as the device code, on the host)
  constexpr bool copy = !std::is_same<T, double>::value;
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
  return TMK_OK;
}

// Scratch of one patch's step -- WM, WP (3 each) | WH1 (3) | WH2 (6) | WH (3) |
// LG | FF (3) | FP32 copy of U (mixed form) -- from `base` (or only its size
// when base is null).  Returns the bytes used.
template <typename T>
size_t layout3(Step3<T>& g, char* base) {
  using namespace tmk::d3;
  constexpr bool copy = !std::is_same<T, double>::value;
  size_t off = 0;
  auto take = [&](size_t bytes) {
    char* p = base ? base + off : nullptr;
    off += align_up3(bytes);
    return p;
  };
  const size_t cell12 = (size_t)NF * g.S.cells() * sizeof(T);
  for (int d = 0; d < 3; ++d) g.WM[d] = (T*)take(cell12);
  for (int d = 0; d < 3; ++d) g.WP[d] = (T*)take(cell12);
  for (int d = 0; d < 3; ++d) g.WH1[d] = (T*)take((size_t)NF * g.fl1[d].cells() * sizeof(T));
  for (int d1 = 0; d1 < 3; ++d1)
    for (int d2 = 0; d2 < 3; ++d2)
      if (d1 != d2) g.WH2[d1][d2] = (T*)take((size_t)NF * g.fl1[d1].cells() * sizeof(T));
  for (int d = 0; d < 3; ++d) g.WH[d] = (T*)take((size_t)NF * g.flF[d].cells() * sizeof(T));
  g.LG = (double*)take(2 * (size_t)g.fplane.cells() * sizeof(double));
  for (int k = 0; k < 3; ++k) g.FF[k] = (double*)take((size_t)TMK_NCOMP * g.fplane.cells() * sizeof(double));
  T* up = (T*)take(copy ? (size_t)NS * g.Ap.cells() * sizeof(T) : 0);
  if constexpr (copy) { g.Up = up; g.Uc = up; g.uside = tmk::NSIDE; }
  else { g.Up = (const T*)(const void*)g.U; g.Uc = nullptr; g.Ap = g.A; g.uside = 11; }
  return off;
}

tmk_status ensure_scratch(tmk_context* c, size_t total, cudaStream_t s) {
  if (total <= c->scratch_bytes) return TMK_OK;
  TMK_CU(cudaStreamSynchronize(s));
  cudaFree(c->scratch);
  c->scratch = nullptr; c->scratch_bytes = 0;
  if (cudaMalloc(&c->scratch, total) != cudaSuccess) return TMK_ERR_ALLOC;
  c->scratch_bytes = total;
  return TMK_OK;
}

// the side stream and events of the overlapped schedule, made once per context
tmk_status ensure_side(tmk_context* c, tmk::d3::Side& side) {
  if (!c->side) {
    cudaStream_t ss = nullptr;
    if (cudaStreamCreateWithFlags(&ss, cudaStreamNonBlocking) != cudaSuccess) return TMK_ERR_CUDA;
    c->side = ss;
    for (int q = 0; q < 6; ++q)
      if (cudaEventCreateWithFlags(&c->side_ev[q], cudaEventDisableTiming) != cudaSuccess) return TMK_ERR_CUDA;
  }
  side.s = c->side;
  for (int q = 0; q < 6; ++q) side.ev[q] = c->side_ev[q];
  return TMK_OK;
}

template <typename T>
tmk_status patch3(tmk_context* c, const tmk_fab3* U, const tmk_fab3* B, const tmk_fab3* const* Fo,
                  const tmk_box3* valid, const tmk_box3* domain, double dx, double time, double dt,
                  cudaStream_t s) {
  using namespace tmk::d3;
  PlanOne<T> pl;
  tmk_status r = fill3<T>(c, U, B, Fo, valid, domain, dx, time, dt, pl.g);
  if (r != TMK_OK) return r;
  if ((r = ensure_scratch(c, layout3<T>(pl.g, nullptr), s)) != TMK_OK) return r;
  layout3<T>(pl.g, (char*)c->scratch);
  Side side;
  if (pl.g.fault && (r = ensure_side(c, side)) != TMK_OK) return r;
  cudaError_t e;
  if constexpr (std::is_same<T, double>::value) e = launch_one_f64(pl, c->dp, c->dstatus, s, &side);
  else e = launch_one_f32(pl, c->dp, c->dstatus, s, &side);
  return e == cudaSuccess ? TMK_OK : TMK_ERR_CUDA;
}

// The patches of a level: their descriptors and each pass's prefix sums in
// the scratch's head, uploaded with one copy, then one launch per pass over
// every patch.
template <typename T>
tmk_status patches3(tmk_context* c, int np, const tmk_fab3* U, const tmk_fab3* B, const tmk_fab3* const* Fa,
                    const tmk_box3* valid, const tmk_box3* domain, double dx, double time, double dt,
                    cudaStream_t s) {
  using namespace tmk::d3;
  std::vector<Step3<T>> gs(np);
  for (int p = 0; p < np; ++p) {
    const tmk_fab3* Fo[3] = {Fa[0] ? Fa[0] + p : nullptr, Fa[1] ? Fa[1] + p : nullptr, Fa[2] ? Fa[2] + p : nullptr};
    const tmk_status r = fill3<T>(c, U + p, B ? B + p : nullptr, Fo, valid + p, domain, dx, time, dt, gs[p]);
    if (r != TMK_OK) return r;
  }
  PlanMany<T> pl;
  pl.np = np;
  pl.copy_ = !std::is_same<T, double>::value;
  pl.fault_ = false;
  for (int d = 0; d < 3; ++d) pl.flux_[d] = false;
  std::vector<long long> start((size_t)NKIND * (np + 1), 0);
  for (int k = 0; k < NKIND; ++k) {
    long long* st = start.data() + (size_t)k * (np + 1);
    for (int p = 0; p < np; ++p) st[p + 1] = st[p] + kind_count(gs[p], k);
    pl.tot[k] = st[np];
  }
  const size_t head = align_up3(np * sizeof(Step3<T>)) + align_up3(start.size() * sizeof(long long));
  size_t total = head;
  std::vector<size_t> offs(np);
  for (int p = 0; p < np; ++p) {
    offs[p] = total;
    total += layout3<T>(gs[p], nullptr);
    pl.fault_ = pl.fault_ || gs[p].fault;
    for (int d = 0; d < 3; ++d) pl.flux_[d] = pl.flux_[d] || gs[p].F[d];
  }
  tmk_status r = ensure_scratch(c, total, s);
  if (r != TMK_OK) return r;
  char* base = (char*)c->scratch;
  for (int p = 0; p < np; ++p) layout3<T>(gs[p], base + offs[p]);
  // descriptors and prefix sums: one upload (pageable: staged before the call returns)
  std::vector<char> hbuf(head);
  std::memcpy(hbuf.data(), gs.data(), np * sizeof(Step3<T>));
  const size_t soff = align_up3(np * sizeof(Step3<T>));
  std::memcpy(hbuf.data() + soff, start.data(), start.size() * sizeof(long long));
  TMK_CU(cudaMemcpyAsync(base, hbuf.data(), head, cudaMemcpyHostToDevice, s));
  pl.dgs = (const Step3<T>*)base;
  pl.dstart = (const long long*)(base + soff);
  Side side;
  if (pl.fault_ && (r = ensure_side(c, side)) != TMK_OK) return r;
  cudaError_t e;
  if constexpr (std::is_same<T, double>::value) e = launch_many_f64(pl, c->dp, c->dstatus, s, &side);
  else e = launch_many_f32(pl, c->dp, c->dstatus, s, &side);
  return e == cudaSuccess ? TMK_OK : TMK_ERR_CUDA;
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

extern "C" tmk_status tmk_patches_update_state_3d(tmk_context* c, int npatch, const tmk_fab3* U, const tmk_fab3* B,
                                                  const tmk_fab3* F0, const tmk_fab3* F1, const tmk_fab3* F2,
                                                  const tmk_box3* valid, const tmk_box3* domain, double dx,
                                                  double time, double dt, double* max_wave_speed, void* stream) {
  if (!c || npatch < 1 || !U || !valid || !domain || !(dx > 0) || !(dt > 0)) return TMK_ERR_BAD_DESC;
  const tmk_fab3* Fa[3] = {F0, F1, F2};
  cudaStream_t s = (cudaStream_t)stream;
  const tmk_status r = c->scheme.precision == TMK_PREC_MIXED
                           ? patches3<float>(c, npatch, U, B, Fa, valid, domain, dx, time, dt, s)
                           : patches3<double>(c, npatch, U, B, Fa, valid, domain, dx, time, dt, s);
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
