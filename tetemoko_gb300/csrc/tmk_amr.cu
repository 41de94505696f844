// tmk_amr.cu -- coarse-fine coupling of device levels and the subcycled AMR
// hierarchy (compiled without FMA contraction: the FP64 form matches the CPU
// oracle's operation order exactly).
//
// A CFLink couples a level (fine side) with the next coarser level.  Built once
// on the host from the two box layouts, it holds device work lists for:
//   * the coarse-fine ghost fill of U (Chombo PiecewiseLinearFillPatch with
//     interpolation radius 4, srcLinElast/LinElastLevelGodunov.cpp:154-160,
//     260-264) and of the fault rows (srcLinElast/D1PiecewiseLinearFillPatch.cpp),
//     as "sites" (coarse cells: time-interpolated value + limited slopes) and
//     "fine entries" (ghost cells: site value + linear terms);
//   * the flux register (Chombo LevelFluxRegister, LinElastLevelGodunov.cpp:
//     334-355): the coarse and fine faces of every coarse-fine face, captured
//     by the volume kernel of each level into its `cap` buffer, and the reflux
//     of AMRLevelLinElast::postTimeStep (:505-506);
//   * average-down (Chombo CoarseAverage; srcLinElast/D1CoarseAverage.cpp with
//     d1average, tetemoko_chombo_patchfile:141-188);
//   * regrid prolongation (Chombo FineInterp; srcLinElast/D1FineInterp.cpp).
// Every list is laid out so that one thread owns one (item, component) and
// writes distinct addresses: no atomics, results independent of scheduling.
// Threads run component-major (neighbouring threads take neighbouring items
// of one component plane), so their state accesses coalesce along x.
#include <cuda_runtime.h>
#include <algorithm>
#include <cmath>
#include <map>
#include <new>
#include <tuple>
#include <vector>

#include "tmk_internal.h"

using tmk::PatchDev;
using tmk::TileDev;
using tmk::CopyDev;
using tmk::fab_idx;
using namespace tmk_host;

namespace {

constexpr int NC = TMK_NCOMP;
constexpr int NG = TMK_NGHOST;

// slope kinds: centred, one-sided towards lo (u0 - u[-1]), towards hi (u[+1] - u0), none
enum { SL_CENTRED = 0, SL_LO = 1, SL_HI = 2, SL_NONE = 3 };

struct SiteU { int ci, cj; int nb[9]; int kx, ky, lim; };   // nb[(dj+1)*3+(di+1)]: coarse patch or -1
struct FineU { int fpatch, i, j, site; double cx, cy; };
struct SiteB { int ci; int nb[3]; int kind; };
struct FineB { int fpatch, i, site; double cx; };
struct AvgU { int cpatch, ci, cj, fpatch; };
struct AvgB { int cpatch, ci, fpatch; };
struct InterpU { int fpatch, ci, cj; int nb[9]; int kx, ky, lim; };
struct InterpB { int fpatch, ci; int nb[3]; int kind, lim; };
struct RefluxCell { int cpatch, ci, cj, e0, e1; };

int cdiv(int i, int r) { return i >= 0 ? i / r : -((-i + r - 1) / r); }
tmk_box coarsen(const tmk_box& b, int r) {
  tmk_box c;
  c.lo[0] = cdiv(b.lo[0], r); c.lo[1] = cdiv(b.lo[1], r);
  c.hi[0] = cdiv(b.hi[0], r); c.hi[1] = cdiv(b.hi[1], r);
  return c;
}

// ------------------------------------------------------------- device code
// The state transfers compute in the state's own type R (FP32 in the mixed
// form: GB300's FP64 rate would dominate these bulk passes; FP64 in the plain
// form, where they match the oracle to rounding).  Fault rows stay FP64.
template <typename R> __device__ __forceinline__ R dmin(R a, R b) { return (b < a) ? b : a; }
template <typename R> __device__ __forceinline__ R dmax(R a, R b) { return (a < b) ? b : a; }

// new*a + old*(1-a); exact copies at a = 1 and a = 0
template <typename R>
__device__ __forceinline__ R tinterp(R o, R n, R a) {
  if (a == R(1)) return n;
  if (a == R(0)) return o;
  R v = n * a;
  R t = o * (R(1) - a);
  return v + t;
}

template <typename R>
__device__ __forceinline__ R slope(int kind, R um, R u0, R up) {
  return kind == SL_CENTRED ? R(0.5) * (up - um) : kind == SL_LO ? u0 - um : kind == SL_HI ? up - u0 : R(0);
}

template <typename R>
__device__ __forceinline__ void limit2(R& sx, R& sy, R u, R mn, R mx) {
  R dm = R(0.5) * (fabs(sx) + fabs(sy));
  R th = R(1);
  if (dm > R(0)) {
    th = dmin(th, (mx - u) / dm);
    th = dmin(th, (u - mn) / dm);
  }
  sx = sx * th;
  sy = sy * th;
}

__device__ __forceinline__ double icoef(int f, int c, int r) { return -0.5 + ((double)(f - r * c) + 0.5) / (double)r; }

template <typename Real>
__device__ __forceinline__ Real uval(const PatchDev<Real>& P, int c, int i, int j, Real a) {
  const size_t o = fab_idx(P, c, i, j);
  const Real n = P.Uin[o];
  if (a == Real(1)) return n;
  return tinterp(P.Uout[o], n, a);
}

__device__ __forceinline__ double bval(const double* B, int blo, int bnx, int c, int i) {
  return B[(size_t)c * bnx + (i - blo)];
}

// coarse sites: time-interpolated value and limited slopes, 3 values per
// (site, comp) in the state's type, 2 doubles per (fault site, comp)
template <typename Real>
__global__ void cf_sites_kernel(const PatchDev<Real>* __restrict__ cp, const SiteU* __restrict__ su, int nsu,
                                const SiteB* __restrict__ sb, int nsb, int nb, double a,
                                Real* __restrict__ svu, double* __restrict__ svb) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < nsu * NC) {                      // component-major: neighbouring threads, neighbouring sites
    const SiteU s = su[t % nsu];
    const int c = t / nsu;
    const Real ar = (Real)a;
    Real v[9];
#pragma unroll
    for (int k = 0; k < 9; ++k)
      v[k] = s.nb[k] >= 0 ? uval(cp[s.nb[k]], c, s.ci + k % 3 - 1, s.cj + k / 3 - 1, ar) : Real(0);
    const Real u0 = v[4];
    Real sx = slope(s.kx, v[3], u0, v[5]);
    Real sy = slope(s.ky, v[1], u0, v[7]);
    if (s.lim) {
      Real mn = u0, mx = u0;
#pragma unroll
      for (int k = 0; k < 9; ++k)
        if (s.nb[k] >= 0) { mn = dmin(mn, v[k]); mx = dmax(mx, v[k]); }
      limit2(sx, sy, u0, mn, mx);
    }
    Real* o = svu + ((size_t)(t % nsu) * NC + c) * 3;
    o[0] = u0; o[1] = sx; o[2] = sy;
    return;
  }
  t -= nsu * NC;
  if (t < nsb * nb) {
    const SiteB s = sb[t % nsb];
    const int c = t / nsb;
    double v[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      v[k] = 0.0;
      if (s.nb[k] < 0) continue;
      const PatchDev<Real>& P = cp[s.nb[k]];
      const int i = s.ci + k - 1;
      const double n = bval(P.B, P.blo0, P.bnx, c, i);
      v[k] = a == 1.0 ? n : tinterp<double>(bval(P.Bold, P.blo0, P.bnx, c, i), n, a);
    }
    double* o = svb + ((size_t)(t % nsb) * nb + c) * 2;
    o[0] = v[1];
    o[1] = slope<double>(s.kind, v[0], v[1], v[2]);
  }
}

// fine ghost cells: site value + linear terms (x first, then y)
template <typename Real>
__global__ void cf_apply_kernel(const PatchDev<Real>* __restrict__ fp, const FineU* __restrict__ fu, int nfu,
                                const FineB* __restrict__ fb, int nfb, int nb,
                                const Real* __restrict__ svu, const double* __restrict__ svb) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < nfu * NC) {
    const FineU e = fu[t % nfu];
    const int c = t / nfu;
    const Real* s = svu + ((size_t)e.site * NC + c) * 3;
    Real v = s[0];
    v = v + (Real)e.cx * s[1];
    v = v + (Real)e.cy * s[2];
    const PatchDev<Real>& P = fp[e.fpatch];
    ((Real*)P.Uin)[fab_idx(P, c, e.i, e.j)] = v;
    return;
  }
  t -= nfu * NC;
  if (t < nfb * nb) {
    const FineB e = fb[t % nfb];
    const int c = t / nfb;
    const double* s = svb + ((size_t)e.site * nb + c) * 2;
    double v = s[0];
    v = v + e.cx * s[1];
    const PatchDev<Real>& P = fp[e.fpatch];
    P.B[(size_t)c * P.bnx + (e.i - P.blo0)] = v;
  }
}

// fault data at the start of a step (AMRLevelLinElast::advance m_BOld.copy)
template <typename Real>
__global__ void bsnap_kernel(const PatchDev<Real>* __restrict__ pd, const int* __restrict__ fpatches, int nb) {
  const PatchDev<Real>& P = pd[fpatches[blockIdx.x]];
  const int n = nb * P.bnx;
  for (int k = threadIdx.x; k < n; k += blockDim.x) P.Bold[k] = P.B[k];
}

// LevelFluxRegister::incrementCoarse: R = -dt * F_coarse
__global__ void reg_coarse_kernel(const double* __restrict__ cap, const int* __restrict__ cslot, int nent, double dt,
                                  double* __restrict__ R) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nent * NC) return;
  const int e = t / NC, c = t % NC;
  R[t] = -(dt * cap[(size_t)cslot[e] * NC + c]);
}

// LevelFluxRegister::incrementFine: R += (dt / r) * F_fine over the r fine faces
__global__ void reg_fine_kernel(const double* __restrict__ cap, const int* __restrict__ fslot, int nent, int r,
                                double s, double* __restrict__ R) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nent * NC) return;
  const int e = t / NC, c = t % NC;
  double v = R[t];
  for (int m = 0; m < r; ++m) v = v + s * cap[(size_t)fslot[e * r + m] * NC + c];
  R[t] = v;
}

// LevelFluxRegister::reflux: each coarse cell applies its entries in order
template <typename Real>
__global__ void reflux_kernel(const PatchDev<Real>* __restrict__ cp, const RefluxCell* __restrict__ cells, int ncells,
                              const int* __restrict__ list, const double* __restrict__ sc,
                              const double* __restrict__ R) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ncells * NC) return;
  const RefluxCell cl = cells[t % ncells];
  const int c = t / ncells;
  const PatchDev<Real>& P = cp[cl.cpatch];
  Real* U = (Real*)P.Uin;
  const size_t o = fab_idx(P, c, cl.ci, cl.cj);
  double v = (double)U[o];
  for (int k = cl.e0; k < cl.e1; ++k) {
    const int e = list[k];
    v = v + R[(size_t)e * NC + c] * sc[e];
  }
  U[o] = (Real)v;
}

// average-down of U (r x r children, x fastest) and of the fault rows (r children)
template <typename Real>
__global__ void avgdown_kernel(const PatchDev<Real>* __restrict__ cp, const PatchDev<Real>* __restrict__ fp,
                               const AvgU* __restrict__ au, int nau, const AvgB* __restrict__ ab, int nab, int nb,
                               int r, double sU, double sB, int both) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < nau) {                           // one coarse cell, all components: neighbouring threads, neighbouring cells
    const AvgU e = au[t];
    const PatchDev<Real>& F = fp[e.fpatch];
    const PatchDev<Real>& C = cp[e.cpatch];
    const Real* src = F.Uin + fab_idx(F, 0, r * e.ci, r * e.cj);
    const size_t fplane = (size_t)F.anx * F.any, frow = F.anx;
    const size_t o = fab_idx(C, 0, e.ci, e.cj), cplane = (size_t)C.anx * C.any;
    const Real s = (Real)sU;
#pragma unroll 2
    for (int c = 0; c < NC; ++c) {
      Real sum = Real(0);
      if (r == 2) {                        // the common ratio: four independent loads
        const Real* q = src + c * fplane;
        sum = sum + q[0]; sum = sum + q[1]; sum = sum + q[frow]; sum = sum + q[frow + 1];
      } else {
        for (int jj = 0; jj < r; ++jj)
          for (int ii = 0; ii < r; ++ii) sum = sum + src[c * fplane + jj * frow + ii];
      }
      const Real v = sum * s;
      ((Real*)C.Uin)[o + c * cplane] = v;
      // lambda, gamma: a step without plasticity never rewrites them, keep both buffers equal
      if (both && (c == 9 || c == 10 || c == 20 || c == 21)) C.Uout[o + c * cplane] = v;
    }
    return;
  }
  t -= nau;
  if (t < nab * nb) {
    const AvgB e = ab[t % nab];
    const int c = t / nab;
    const PatchDev<Real>& F = fp[e.fpatch];
    double sum = 0.0;
    for (int ii = 0; ii < r; ++ii) sum = sum + bval(F.B, F.blo0, F.bnx, c, r * e.ci + ii);
    const PatchDev<Real>& C = cp[e.cpatch];
    C.B[(size_t)c * C.bnx + (e.ci - C.blo0)] = sum * sB;
  }
}

// regrid prolongation of valid cells: constant + limited linear, into both buffers
template <typename Real>
__global__ void finterp_kernel(const PatchDev<Real>* __restrict__ cp, const PatchDev<Real>* __restrict__ fp,
                               const InterpU* __restrict__ iu, int niu, const InterpB* __restrict__ ib, int nib,
                               int nb, int r) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < niu * NC) {
    const InterpU e = iu[t % niu];
    const int c = t / niu;
    double v[9];
#pragma unroll
    for (int k = 0; k < 9; ++k)
      v[k] = e.nb[k] >= 0 ? (double)cp[e.nb[k]].Uin[fab_idx(cp[e.nb[k]], c, e.ci + k % 3 - 1, e.cj + k / 3 - 1)]
                          : 0.0;
    const double u0 = v[4];
    double sx = slope(e.kx, v[3], u0, v[5]);
    double sy = slope(e.ky, v[1], u0, v[7]);
    if (e.lim) {
      double mn = u0, mx = u0;
#pragma unroll
      for (int k = 0; k < 9; ++k)
        if (e.nb[k] >= 0) { mn = dmin(mn, v[k]); mx = dmax(mx, v[k]); }
      limit2(sx, sy, u0, mn, mx);
    }
    const PatchDev<Real>& F = fp[e.fpatch];
    for (int jj = 0; jj < r; ++jj)
      for (int ii = 0; ii < r; ++ii) {
        const int i = r * e.ci + ii, j = r * e.cj + jj;
        double w = u0;
        w = w + icoef(i, e.ci, r) * sx;
        w = w + icoef(j, e.cj, r) * sy;
        const size_t o = fab_idx(F, c, i, j);
        ((Real*)F.Uin)[o] = (Real)w;
        F.Uout[o] = (Real)w;
      }
    return;
  }
  t -= niu * NC;
  if (t < nib * nb) {
    const InterpB e = ib[t % nib];
    const int c = t / nib;
    double v[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      v[k] = 0.0;
      if (e.nb[k] >= 0) { const PatchDev<Real>& P = cp[e.nb[k]]; v[k] = bval(P.B, P.blo0, P.bnx, c, e.ci + k - 1); }
    }
    const double u0 = v[1];
    double s = slope(e.kind, v[0], u0, v[2]);
    if (e.lim) {
      double mn = u0, mx = u0;
#pragma unroll
      for (int k = 0; k < 3; ++k) { mn = dmin(mn, v[k]); mx = dmax(mx, v[k]); }
      double s1 = 0.0;
      limit2(s, s1, u0, mn, mx);
    }
    const PatchDev<Real>& F = fp[e.fpatch];
    for (int ii = 0; ii < r; ++ii) {
      const int i = r * e.ci + ii;
      double w = u0;
      w = w + icoef(i, e.ci, r) * s;
      F.B[(size_t)c * F.bnx + (i - F.blo0)] = w;
    }
  }
}

// copy of overlapping valid regions between two levels (regrid), both buffers
template <typename Real>
__global__ void xcopy_kernel(const PatchDev<Real>* __restrict__ dst, const PatchDev<Real>* __restrict__ src,
                             const CopyDev* __restrict__ copies, int nu, int nb) {
  const CopyDev cp = copies[blockIdx.x];
  const PatchDev<Real>& S = src[cp.src];
  const PatchDev<Real>& D = dst[cp.dst];
  const int nx = cp.hi0 - cp.lo0 + 1, ny = cp.hi1 - cp.lo1 + 1;
  if ((int)blockIdx.x < nu) {
    for (int idx = threadIdx.x; idx < NC * nx * ny; idx += blockDim.x) {
      const int c = idx / (nx * ny), j = cp.lo1 + (idx / nx) % ny, i = cp.lo0 + idx % nx;
      const Real v = S.Uin[fab_idx(S, c, i, j)];
      const size_t o = fab_idx(D, c, i, j);
      ((Real*)D.Uin)[o] = v;
      D.Uout[o] = v;
    }
  } else {
    for (int idx = threadIdx.x; idx < nb * nx; idx += blockDim.x) {
      const int c = idx / nx, i = cp.lo0 + idx % nx;
      D.B[(size_t)c * D.bnx + (i - D.blo0)] = bval(S.B, S.blo0, S.bnx, c, i);
    }
  }
}

unsigned blocks_for(long long n, int nt) { return (unsigned)std::max(1LL, (n + nt - 1) / nt); }

template <typename T>
tmk_status upload(std::vector<void*>& allocs, T** dptr, const std::vector<T>& v) {
  *dptr = nullptr;
  if (v.empty()) return TMK_OK;
  if (dalloc(dptr, v.size()) != cudaSuccess) return TMK_ERR_ALLOC;
  allocs.push_back(*dptr);
  TMK_CU(cudaMemcpy(*dptr, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
  return TMK_OK;
}

int patch_at(const tmk_level_s* L, int i, int j) {
  for (size_t p = 0; p < L->patches.size(); ++p)
    if (box_has(L->patches[p].valid, i, j)) return (int)p;
  return -1;
}
int fault_patch_at(const tmk_level_s* L, int i) {
  for (size_t p = 0; p < L->patches.size(); ++p)
    if (L->patches[p].fault && i >= L->patches[p].valid.lo[0] && i <= L->patches[p].valid.hi[0]) return (int)p;
  return -1;
}

}  // namespace

namespace tmk_host {

// a captured face: the patch that computes it, the direction and face index
using FaceKey = std::tuple<int, int, int, int>;   // (patch, dir, i, j)

struct CFLink {
  tmk_level_s* F = nullptr;
  tmk_level_s* C = nullptr;
  int r = 1;
  std::vector<void*> allocs;
  // coarse-fine ghost fill
  SiteU* dsu = nullptr; int nsu = 0;
  FineU* dfu = nullptr; int nfu = 0;
  SiteB* dsb = nullptr; int nsb = 0;
  FineB* dfb = nullptr; int nfb = 0;
  double* dsvu = nullptr;
  double* dsvb = nullptr;
  // flux register
  int nent = 0;
  std::vector<FaceKey> cface;        // per entry, captured by C
  std::vector<FaceKey> fface;        // r per entry, captured by F
  int* dcslot = nullptr;
  int* dfslot = nullptr;
  double* dR = nullptr;
  RefluxCell* dcells = nullptr; int ncells = 0;
  int* dlist = nullptr;
  double* dsc = nullptr;
  // average-down and prolongation
  AvgU* dau = nullptr; int nau = 0;
  AvgB* dab = nullptr; int nab = 0;
  InterpU* diu = nullptr; int niu = 0;
  InterpB* dib = nullptr; int nib = 0;
  ~CFLink() { for (void* p : allocs) cudaFree(p); }
};

}  // namespace tmk_host

namespace {

// Assign capture slots to the faces that the level's links need, group them
// by the tile that computes them, and refresh the links' slot tables.
tmk_status rebuild_captures_impl(tmk_level_s* L) {
  std::map<FaceKey, int> slot;
  if (L->coarser) for (const FaceKey& k : L->coarser->fface) slot.emplace(k, 0);
  if (L->finer) for (const FaceKey& k : L->finer->cface) slot.emplace(k, 0);
  int n = 0;
  for (auto& kv : slot) kv.second = n++;
  // owning tile of each face: x face i belongs to the tile holding cell i (the
  // patch's last hi face to its last tile), likewise for y faces
  std::vector<std::vector<int4>> per_tile(L->htiles.size());
  for (const auto& kv : slot) {
    const int p = std::get<0>(kv.first), d = std::get<1>(kv.first);
    const int i = std::get<2>(kv.first), j = std::get<3>(kv.first);
    const tmk_box& v = L->patches[p].valid;
    const int ci = d == 0 ? std::min(i, v.hi[0]) : i, cj = d == 1 ? std::min(j, v.hi[1]) : j;
    int owner = -1;
    for (size_t t = 0; t < L->htiles.size(); ++t) {
      const TileDev& tl = L->htiles[t];
      if (tl.patch == p && ci >= tl.x0 && ci < tl.x0 + tl.nx && cj >= tl.y0 && cj < tl.y0 + tl.ny) { owner = (int)t; break; }
    }
    if (owner < 0) return TMK_ERR_BAD_DESC;
    per_tile[owner].push_back(make_int4(d, i, j, kv.second));
  }
  std::vector<int4> list;
  for (size_t t = 0; t < L->htiles.size(); ++t) {
    L->htiles[t].cap0 = (int)list.size();
    L->htiles[t].ncap = (int)per_tile[t].size();
    list.insert(list.end(), per_tile[t].begin(), per_tile[t].end());
  }
  TMK_CU(cudaDeviceSynchronize());
  for (void* p : L->cap_allocs) cudaFree(p);
  L->cap_allocs.clear();
  L->cap = nullptr; L->dcaplist = nullptr; L->ncap = n;
  L->dmcap[0] = L->dmcap[1] = nullptr;
  if (n) {
    if (dalloc(&L->cap, (size_t)n * NC) != cudaSuccess) return TMK_ERR_ALLOC;
    L->cap_allocs.push_back(L->cap);
    TMK_CU(cudaMemset(L->cap, 0, (size_t)n * NC * sizeof(double)));
    if (dalloc(&L->dcaplist, list.size()) != cudaSuccess) return TMK_ERR_ALLOC;
    L->cap_allocs.push_back(L->dcaplist);
    TMK_CU(cudaMemcpy(L->dcaplist, list.data(), list.size() * sizeof(int4), cudaMemcpyHostToDevice));
  }
  TMK_CU(cudaMemcpy(L->dtiles, L->htiles.data(), L->htiles.size() * sizeof(TileDev), cudaMemcpyHostToDevice));
  // the same faces for the marching items of each component group: the item
  // holding the cell on the face's side inside the patch, sorted by row
  for (int g = 0; g < 2 && L->march_allowed; ++g) {
    std::vector<tmk::MarchItem>& items = L->hitems[g];
    std::vector<std::vector<int4>> per(items.size());
    for (const auto& kv : slot) {
      const int p = std::get<0>(kv.first), d = std::get<1>(kv.first);
      const int i = std::get<2>(kv.first), j = std::get<3>(kv.first);
      const tmk_box& v = L->patches[p].valid;
      int ci = i, cj = j, kind;
      if (d == 0) { kind = i <= v.hi[0] ? 0 : 1; if (kind == 1) ci = i - 1; }
      else { kind = j <= v.hi[1] ? 2 : 3; if (kind == 3) cj = j - 1; }
      int owner = -1;
      for (size_t k = 0; k < items.size(); ++k) {
        const tmk::MarchItem& m = items[k];
        if (m.patch == p && ci >= m.x0 && ci < m.x0 + tmk::MARCH_COLS && cj >= m.y0 && cj <= m.y1) { owner = (int)k; break; }
      }
      if (owner < 0) return TMK_ERR_BAD_DESC;
      per[owner].push_back(make_int4(cj, kind, ci - items[owner].x0 + tmk::MARCH_HALO, kv.second));
    }
    std::vector<int4> caps;
    for (size_t k = 0; k < items.size(); ++k) {
      std::stable_sort(per[k].begin(), per[k].end(), [](const int4& a, const int4& b) { return a.x < b.x; });
      items[k].cap0 = (int)caps.size();
      items[k].ncap = (int)per[k].size();
      caps.insert(caps.end(), per[k].begin(), per[k].end());
    }
    for (tmk::MarchItem& f : L->hfrows[g])
      for (const tmk::MarchItem& m : items)
        if (m.patch == f.patch && m.x0 == f.x0 && m.y0 == f.y0) { f.cap0 = m.cap0; f.ncap = m.ncap; break; }
    L->dmcap[g] = nullptr;
    if (!caps.empty()) {
      if (dalloc(&L->dmcap[g], caps.size()) != cudaSuccess) return TMK_ERR_ALLOC;
      L->cap_allocs.push_back(L->dmcap[g]);
      TMK_CU(cudaMemcpy(L->dmcap[g], caps.data(), caps.size() * sizeof(int4), cudaMemcpyHostToDevice));
    }
    TMK_CU(cudaMemcpy(L->ditems[g], items.data(), items.size() * sizeof(tmk::MarchItem), cudaMemcpyHostToDevice));
    if (!L->hfrows[g].empty())
      TMK_CU(cudaMemcpy(L->dfrows[g], L->hfrows[g].data(), L->hfrows[g].size() * sizeof(tmk::MarchItem),
                        cudaMemcpyHostToDevice));
  }
  L->march = L->march_allowed && L->tune.volume_kernel == TMK_VOLUME_MARCH;
  if (upload_patchdev(L, 0) != TMK_OK) return TMK_ERR_CUDA;
  // slot tables of the links that use this level's captures
  if (L->coarser && L->coarser->nent) {
    std::vector<int> fs;
    for (const FaceKey& k : L->coarser->fface) fs.push_back(slot[k]);
    TMK_CU(cudaMemcpy(L->coarser->dfslot, fs.data(), fs.size() * sizeof(int), cudaMemcpyHostToDevice));
  }
  if (L->finer && L->finer->nent) {
    std::vector<int> cs;
    for (const FaceKey& k : L->finer->cface) cs.push_back(slot[k]);
    TMK_CU(cudaMemcpy(L->finer->dcslot, cs.data(), cs.size() * sizeof(int), cudaMemcpyHostToDevice));
  }
  TMK_CU(cudaDeviceSynchronize());
  return TMK_OK;
}

void free_link(CFLink* k) {
  if (!k) return;
  cudaDeviceSynchronize();
  delete k;
}

// Unlink level F from its coarser level (both sides' captures are rebuilt).
void detach(tmk_level_s* F) {
  CFLink* k = F->coarser;
  if (!k) return;
  tmk_level_s* C = k->C;
  F->coarser = nullptr;
  if (C && C->finer == k) C->finer = nullptr;
  free_link(k);
  rebuild_captures_impl(F);
  if (C) rebuild_captures_impl(C);
}

tmk_status build_link(CFLink* k) {
  tmk_level_s* F = k->F;
  tmk_level_s* C = k->C;
  const int r = k->r;
  const int nb = F->ctx->nb;
  const tmk_box& fdom = F->domain;
  const tmk_box& cdom = C->domain;
  std::vector<tmk_box> cfb;
  for (const LevelPatch& lp : F->patches) cfb.push_back(coarsen(lp.valid, r));
  auto covered_by_fine = [&](int ci, int cj) {
    for (const tmk_box& b : cfb) if (box_has(b, ci, cj)) return true;
    return false;
  };
  auto covered_by_fine_row = [&](int ci) {
    for (size_t q = 0; q < F->patches.size(); ++q)
      if (F->patches[q].fault && ci >= cfb[q].lo[0] && ci <= cfb[q].hi[0]) return true;
    return false;
  };
  // ---- coarse-fine ghost fill of U
  std::vector<SiteU> su;
  std::vector<FineU> fu;
  std::map<std::pair<int, int>, int> site_of;
  for (size_t p = 0; p < F->patches.size(); ++p) {
    const tmk_box& V = F->patches[p].valid;
    const tmk_box g = box_isect(box_grow(V, NG), fdom);
    for (int j = g.lo[1]; j <= g.hi[1]; ++j)
      for (int i = g.lo[0]; i <= g.hi[0]; ++i) {
        if (box_has(V, i, j)) continue;
        const int ci = cdiv(i, r), cj = cdiv(j, r);
        if (covered_by_fine(ci, cj)) continue;
        if (patch_at(C, ci, cj) < 0) return TMK_ERR_BAD_DESC;   // not properly nested
        auto it = site_of.find({ci, cj});
        int sidx;
        if (it == site_of.end()) {
          SiteU s;
          s.ci = ci; s.cj = cj;
          for (int k9 = 0; k9 < 9; ++k9) s.nb[k9] = patch_at(C, ci + k9 % 3 - 1, cj + k9 / 3 - 1);
          const bool xm = s.nb[3] >= 0, xp = s.nb[5] >= 0, ym = s.nb[1] >= 0, yp = s.nb[7] >= 0;
          s.kx = (xm && xp) ? SL_CENTRED : xm ? SL_LO : xp ? SL_HI : SL_NONE;
          s.ky = (ym && yp) ? SL_CENTRED : ym ? SL_LO : yp ? SL_HI : SL_NONE;
          tmk_box one; one.lo[0] = ci - 1; one.lo[1] = cj - 1; one.hi[0] = ci + 1; one.hi[1] = cj + 1;
          s.lim = box_contains(cdom, one) ? 1 : 0;
          sidx = (int)su.size();
          su.push_back(s);
          site_of[{ci, cj}] = sidx;
        } else {
          sidx = it->second;
        }
        FineU e;
        e.fpatch = (int)p; e.i = i; e.j = j; e.site = sidx;
        e.cx = -0.5 + ((double)(i - r * ci) + 0.5) / (double)r;
        e.cy = -0.5 + ((double)(j - r * cj) + 0.5) / (double)r;
        fu.push_back(e);
      }
  }
  // ---- coarse-fine ghost fill of the fault rows
  std::vector<SiteB> sb;
  std::vector<FineB> fb;
  std::map<int, int> bsite_of;
  if (nb > 0)
    for (size_t p = 0; p < F->patches.size(); ++p) {
      if (!F->patches[p].fault) continue;
      const tmk_box& V = F->patches[p].valid;
      const int lo = std::max(V.lo[0] - NG, fdom.lo[0]), hi = std::min(V.hi[0] + NG, fdom.hi[0]);
      for (int i = lo; i <= hi; ++i) {
        if (i >= V.lo[0] && i <= V.hi[0]) continue;
        const int ci = cdiv(i, r);
        if (covered_by_fine_row(ci)) continue;
        if (fault_patch_at(C, ci) < 0) return TMK_ERR_BAD_DESC;
        auto it = bsite_of.find(ci);
        int sidx;
        if (it == bsite_of.end()) {
          SiteB s;
          s.ci = ci;
          for (int k3 = 0; k3 < 3; ++k3) s.nb[k3] = fault_patch_at(C, ci + k3 - 1);
          const bool hm = s.nb[0] >= 0, hp = s.nb[2] >= 0;
          s.kind = (hm && hp) ? SL_CENTRED : hm ? SL_LO : hp ? SL_HI : SL_NONE;
          sidx = (int)sb.size();
          sb.push_back(s);
          bsite_of[ci] = sidx;
        } else {
          sidx = it->second;
        }
        FineB e;
        e.fpatch = (int)p; e.i = i; e.site = sidx;
        e.cx = -0.5 + ((double)(i - r * ci) + 0.5) / (double)r;
        fb.push_back(e);
      }
    }
  // ---- flux register: entries in the order d, side (lo, hi), fine patch, tangential
  struct Ent { int q, ci, cj, side; };
  std::vector<Ent> ents;
  for (int d = 0; d < 2; ++d)
    for (int side = -1; side <= 1; side += 2)
      for (size_t p = 0; p < F->patches.size(); ++p) {
        const tmk_box& vc = cfb[p];
        const tmk_box& V = F->patches[p].valid;
        const int t = 1 - d;
        const int kd = side < 0 ? vc.lo[d] - 1 : vc.hi[d] + 1;
        for (int kt = vc.lo[t]; kt <= vc.hi[t]; ++kt) {
          const int ci = d == 0 ? kd : kt, cj = d == 0 ? kt : kd;
          if (!box_has(cdom, ci, cj) || covered_by_fine(ci, cj)) continue;
          const int q = patch_at(C, ci, cj);
          if (q < 0) return TMK_ERR_BAD_DESC;
          const int cf = kd + (side < 0 ? 1 : 0);
          k->cface.emplace_back(q, d, d == 0 ? cf : ci, d == 0 ? cj : cf);
          const int ff = side < 0 ? V.lo[d] : V.hi[d] + 1;
          for (int m = 0; m < r; ++m) {
            const int tt = r * kt + m;
            k->fface.emplace_back((int)p, d, d == 0 ? ff : tt, d == 0 ? tt : ff);
          }
          ents.push_back({q, ci, cj, side});
        }
      }
  k->nent = (int)ents.size();
  // reflux: entries grouped by coarse cell, each cell's entries in register order
  std::map<std::tuple<int, int, int>, std::vector<int>> by_cell;
  for (int e = 0; e < k->nent; ++e) by_cell[std::make_tuple(ents[e].q, ents[e].ci, ents[e].cj)].push_back(e);
  std::vector<RefluxCell> cells;
  std::vector<int> list;
  for (const auto& kv : by_cell) {
    RefluxCell rc;
    rc.cpatch = std::get<0>(kv.first); rc.ci = std::get<1>(kv.first); rc.cj = std::get<2>(kv.first);
    rc.e0 = (int)list.size();
    list.insert(list.end(), kv.second.begin(), kv.second.end());
    rc.e1 = (int)list.size();
    cells.push_back(rc);
  }
  const double scale = -1.0 / C->dx;
  std::vector<double> sc;
  for (const Ent& e : ents) sc.push_back(e.side < 0 ? scale : -scale);
  // ---- average-down and prolongation lists
  std::vector<AvgU> au;
  std::vector<AvgB> ab;
  std::vector<InterpU> iu;
  std::vector<InterpB> ib;
  for (size_t p = 0; p < F->patches.size(); ++p) {
    const tmk_box& vc = cfb[p];
    for (int cj = vc.lo[1]; cj <= vc.hi[1]; ++cj)
      for (int ci = vc.lo[0]; ci <= vc.hi[0]; ++ci) {
        const int q = patch_at(C, ci, cj);
        if (q < 0) return TMK_ERR_BAD_DESC;
        au.push_back({q, ci, cj, (int)p});
        InterpU e;
        e.fpatch = (int)p; e.ci = ci; e.cj = cj;
        for (int k9 = 0; k9 < 9; ++k9) e.nb[k9] = patch_at(C, ci + k9 % 3 - 1, cj + k9 / 3 - 1);
        int kind[2];
        for (int d = 0; d < 2; ++d) {
          const int cd = d == 0 ? ci : cj;
          const bool atlo = cd == cdom.lo[d], athi = cd == cdom.hi[d];
          kind[d] = (!atlo && !athi) ? SL_CENTRED : (atlo && !athi) ? SL_HI : (athi && !atlo) ? SL_LO : SL_NONE;
          const int kp = d == 0 ? 5 : 7, km = d == 0 ? 3 : 1;
          if ((kind[d] == SL_CENTRED || kind[d] == SL_HI) && e.nb[kp] < 0) return TMK_ERR_BAD_DESC;
          if ((kind[d] == SL_CENTRED || kind[d] == SL_LO) && e.nb[km] < 0) return TMK_ERR_BAD_DESC;
        }
        e.kx = kind[0]; e.ky = kind[1];
        tmk_box one; one.lo[0] = ci - 1; one.lo[1] = cj - 1; one.hi[0] = ci + 1; one.hi[1] = cj + 1;
        e.lim = box_contains(cdom, one) ? 1 : 0;
        iu.push_back(e);
      }
    if (nb == 0 || !F->patches[p].fault) continue;
    for (int ci = vc.lo[0]; ci <= vc.hi[0]; ++ci) {
      const int q = fault_patch_at(C, ci);
      if (q < 0) return TMK_ERR_BAD_DESC;
      ab.push_back({q, ci, (int)p});
      InterpB e;
      e.fpatch = (int)p; e.ci = ci;
      for (int k3 = 0; k3 < 3; ++k3) e.nb[k3] = fault_patch_at(C, ci + k3 - 1);
      const bool atlo = ci == cdom.lo[0], athi = ci == cdom.hi[0];
      e.kind = (!atlo && !athi) ? SL_CENTRED : (atlo && !athi) ? SL_HI : (athi && !atlo) ? SL_LO : SL_NONE;
      if ((e.kind == SL_CENTRED || e.kind == SL_HI) && e.nb[2] < 0) return TMK_ERR_BAD_DESC;
      if ((e.kind == SL_CENTRED || e.kind == SL_LO) && e.nb[0] < 0) return TMK_ERR_BAD_DESC;
      e.lim = (ci - 1 >= cdom.lo[0] && ci + 1 <= cdom.hi[0]) ? 1 : 0;
      ib.push_back(e);
    }
  }
  // ---- upload
  tmk_status st;
  if ((st = upload(k->allocs, &k->dsu, su)) != TMK_OK) return st;
  if ((st = upload(k->allocs, &k->dfu, fu)) != TMK_OK) return st;
  if ((st = upload(k->allocs, &k->dsb, sb)) != TMK_OK) return st;
  if ((st = upload(k->allocs, &k->dfb, fb)) != TMK_OK) return st;
  k->nsu = (int)su.size(); k->nfu = (int)fu.size(); k->nsb = (int)sb.size(); k->nfb = (int)fb.size();
  if (k->nsu) {
    if (dalloc(&k->dsvu, (size_t)k->nsu * NC * 3) != cudaSuccess) return TMK_ERR_ALLOC;
    k->allocs.push_back(k->dsvu);
  }
  if (k->nsb) {
    if (dalloc(&k->dsvb, (size_t)k->nsb * nb * 2) != cudaSuccess) return TMK_ERR_ALLOC;
    k->allocs.push_back(k->dsvb);
  }
  if (k->nent) {
    if (dalloc(&k->dcslot, (size_t)k->nent) != cudaSuccess || dalloc(&k->dfslot, (size_t)k->nent * r) != cudaSuccess ||
        dalloc(&k->dR, (size_t)k->nent * NC) != cudaSuccess)
      return TMK_ERR_ALLOC;
    k->allocs.push_back(k->dcslot); k->allocs.push_back(k->dfslot); k->allocs.push_back(k->dR);
    TMK_CU(cudaMemset(k->dR, 0, (size_t)k->nent * NC * sizeof(double)));
  }
  if ((st = upload(k->allocs, &k->dcells, cells)) != TMK_OK) return st;
  if ((st = upload(k->allocs, &k->dlist, list)) != TMK_OK) return st;
  if ((st = upload(k->allocs, &k->dsc, sc)) != TMK_OK) return st;
  k->ncells = (int)cells.size();
  if ((st = upload(k->allocs, &k->dau, au)) != TMK_OK) return st;
  if ((st = upload(k->allocs, &k->dab, ab)) != TMK_OK) return st;
  if ((st = upload(k->allocs, &k->diu, iu)) != TMK_OK) return st;
  if ((st = upload(k->allocs, &k->dib, ib)) != TMK_OK) return st;
  k->nau = (int)au.size(); k->nab = (int)ab.size(); k->niu = (int)iu.size(); k->nib = (int)ib.size();
  return TMK_OK;
}

// fault data snapshots for the levels that have a finer level
tmk_status ensure_bold(tmk_level_s* L) {
  for (LevelPatch& lp : L->patches) {
    if (!lp.fault || lp.Bold) continue;
    if (dalloc(&lp.Bold, (size_t)L->ctx->nb * lp.bnx) != cudaSuccess) return TMK_ERR_ALLOC;
    L->allocs.push_back(lp.Bold);
    TMK_CU(cudaMemcpy(lp.Bold, lp.B, (size_t)L->ctx->nb * lp.bnx * sizeof(double), cudaMemcpyDeviceToDevice));
  }
  return TMK_OK;
}

template <typename Real>
tmk_status launch_fill(CFLink* k, double alpha, cudaStream_t s) {
  const int nb = k->F->ctx->nb;
  const long long ns = (long long)k->nsu * NC + (long long)k->nsb * nb;
  const long long nf = (long long)k->nfu * NC + (long long)k->nfb * nb;
  if (ns == 0) return TMK_OK;
  const PatchDev<Real>* cp = (const PatchDev<Real>*)k->C->dpatch[k->C->parity];
  const PatchDev<Real>* fp = (const PatchDev<Real>*)k->F->dpatch[k->F->parity];
  cf_sites_kernel<Real><<<blocks_for(ns, 128), 128, 0, s>>>(cp, k->dsu, k->nsu, k->dsb, k->nsb, nb, alpha,
                                                             (Real*)k->dsvu, k->dsvb);
  TMK_CU(cudaGetLastError());
  cf_apply_kernel<Real><<<blocks_for(nf, 128), 128, 0, s>>>(fp, k->dfu, k->nfu, k->dfb, k->nfb, nb,
                                                             (const Real*)k->dsvu, k->dsvb);
  TMK_CU(cudaGetLastError());
  return TMK_OK;
}

tmk_status fill(CFLink* k, double alpha, cudaStream_t s) {
  return k->F->prec == TMK_PREC_MIXED ? launch_fill<float>(k, alpha, s) : launch_fill<double>(k, alpha, s);
}

template <typename Real>
tmk_status launch_reflux(CFLink* k, cudaStream_t s) {
  if (!k->ncells) return TMK_OK;
  const PatchDev<Real>* cp = (const PatchDev<Real>*)k->C->dpatch[k->C->parity];
  reflux_kernel<Real><<<blocks_for((long long)k->ncells * NC, 128), 128, 0, s>>>(cp, k->dcells, k->ncells,
                                                                                   k->dlist, k->dsc, k->dR);
  TMK_CU(cudaGetLastError());
  return TMK_OK;
}

template <typename Real>
tmk_status launch_avgdown(CFLink* k, cudaStream_t s) {
  const int nb = k->F->ctx->nb;
  const long long n = (long long)k->nau + (long long)k->nab * nb;
  if (!n) return TMK_OK;
  const PatchDev<Real>* cp = (const PatchDev<Real>*)k->C->dpatch[k->C->parity];
  const PatchDev<Real>* fp = (const PatchDev<Real>*)k->F->dpatch[k->F->parity];
  const int r = k->r;
  const int both = k->C->ctx->scheme.plasticity ? 0 : 1;
  avgdown_kernel<Real><<<blocks_for(n, 128), 128, 0, s>>>(cp, fp, k->dau, k->nau, k->dab, k->nab, nb, r,
                                                          1.0 / (double)(r * r), 1.0 / (double)r, both);
  TMK_CU(cudaGetLastError());
  return TMK_OK;
}

template <typename Real>
tmk_status launch_interp(CFLink* k, cudaStream_t s) {
  const int nb = k->F->ctx->nb;
  const long long n = (long long)k->niu * NC + (long long)k->nib * nb;
  if (!n) return TMK_OK;
  const PatchDev<Real>* cp = (const PatchDev<Real>*)k->C->dpatch[k->C->parity];
  const PatchDev<Real>* fp = (const PatchDev<Real>*)k->F->dpatch[k->F->parity];
  finterp_kernel<Real><<<blocks_for(n, 128), 128, 0, s>>>(cp, fp, k->diu, k->niu, k->dib, k->nib, nb, k->r);
  TMK_CU(cudaGetLastError());
  return TMK_OK;
}

double snap_alpha(double time, double dt, double tco, double tcn, int r) {
  double alpha = (time - tco) / (tcn - tco);
  const double eps = 0.04 * dt / r;
  if (std::fabs(alpha) < eps) alpha = 0.0;
  if (std::fabs(1.0 - alpha) < eps) alpha = 1.0;
  return alpha;
}

}  // namespace

// ------------------------------------------------------- level-step hooks
namespace tmk_host {

tmk_status rebuild_captures(tmk_level_s* L) { return rebuild_captures_impl(L); }

tmk_status amr_pre_step(tmk_level_s* L, double time, double dt, double tco, double tcn, cudaStream_t s) {
  if (L->finer && L->nfault && L->ctx->nb > 0) {
    if (L->prec == TMK_PREC_MIXED)
      bsnap_kernel<float><<<L->nfault, 256, 0, s>>>((const PatchDev<float>*)L->dpatch[L->parity], L->dfault,
                                                     L->ctx->nb);
    else
      bsnap_kernel<double><<<L->nfault, 256, 0, s>>>((const PatchDev<double>*)L->dpatch[L->parity], L->dfault,
                                                      L->ctx->nb);
    TMK_CU(cudaGetLastError());
  }
  if (L->coarser) {
    const double alpha = snap_alpha(time, dt, tco, tcn, L->coarser->r);
    if (!(alpha >= 0.0 && alpha <= 1.0)) return TMK_ERR_BAD_DESC;   // LinElastLevelGodunov.cpp:246-256
    return fill(L->coarser, alpha, s);
  }
  return TMK_OK;
}

tmk_status amr_post_step(tmk_level_s* L, double dt, cudaStream_t s) {
  if (L->finer && L->finer->nent) {
    CFLink* k = L->finer;
    reg_coarse_kernel<<<blocks_for((long long)k->nent * NC, 128), 128, 0, s>>>(L->cap, k->dcslot, k->nent, dt, k->dR);
    TMK_CU(cudaGetLastError());
  }
  if (L->coarser && L->coarser->nent) {
    CFLink* k = L->coarser;
    reg_fine_kernel<<<blocks_for((long long)k->nent * NC, 128), 128, 0, s>>>(L->cap, k->dfslot, k->nent, k->r,
                                                                             dt / (double)k->r, k->dR);
    TMK_CU(cudaGetLastError());
  }
  return TMK_OK;
}

int amr_launches(const tmk_level_s* L) {
  int n = 0;
  if (L->finer && L->nfault && L->ctx->nb > 0) ++n;
  if (L->coarser && (L->coarser->nsu || L->coarser->nsb)) n += 2;
  if (L->finer && L->finer->nent) ++n;
  if (L->coarser && L->coarser->nent) ++n;
  return n;
}

void amr_release(tmk_level_s* L) {
  if (L->finer) detach(L->finer->F);
  if (L->coarser) detach(L);
}

}  // namespace tmk_host

// ================================================================= C ABI ===
extern "C" tmk_status tmk_level_attach_coarser(tmk_level* fine, tmk_level* coarse, int ref_ratio) {
  if (!fine || !coarse || fine == coarse || ref_ratio < 2) return TMK_ERR_BAD_DESC;
  if (fine->nscen != 1 || coarse->nscen != 1) return TMK_ERR_UNSUPPORTED;   // ensembles step single levels
  if (fine->graphs || coarse->graphs) return TMK_ERR_BAD_DESC;   // a recorded graph uses their lists
  if (fine->ctx->nb != coarse->ctx->nb || fine->prec != coarse->prec) return TMK_ERR_BAD_DESC;
  const int r = ref_ratio;
  for (int d = 0; d < 2; ++d)
    if (fine->domain.lo[d] != coarse->domain.lo[d] * r || fine->domain.hi[d] != (coarse->domain.hi[d] + 1) * r - 1)
      return TMK_ERR_BAD_DESC;
  if (std::fabs(fine->dx * r - coarse->dx) > 1e-9 * coarse->dx) return TMK_ERR_BAD_DESC;
  for (const LevelPatch& lp : fine->patches)
    for (int d = 0; d < 2; ++d)
      if (lp.valid.lo[d] % r != 0 || (lp.valid.hi[d] + 1) % r != 0) return TMK_ERR_BAD_DESC;
  detach(fine);
  if (coarse->finer) detach(coarse->finer->F);
  CFLink* k = new (std::nothrow) CFLink();
  if (!k) return TMK_ERR_ALLOC;
  k->F = fine; k->C = coarse; k->r = r;
  tmk_status st = build_link(k);
  if (st != TMK_OK) { free_link(k); return st; }
  if ((st = ensure_bold(coarse)) != TMK_OK) { free_link(k); return st; }
  fine->coarser = k;
  coarse->finer = k;
  if ((st = rebuild_captures_impl(fine)) != TMK_OK || (st = rebuild_captures_impl(coarse)) != TMK_OK) {
    detach(fine);
    return st;
  }
  return TMK_OK;
}

extern "C" tmk_status tmk_level_detach_coarser(tmk_level* fine) {
  if (!fine) return TMK_ERR_BAD_DESC;
  if (fine->graphs || (fine->coarser && fine->coarser->C->graphs)) return TMK_ERR_BAD_DESC;
  detach(fine);
  return TMK_OK;
}

extern "C" tmk_status tmk_level_fill_coarse_fine(tmk_level* fine, double alpha, void* stream) {
  if (!fine || !fine->coarser || !(alpha >= 0.0 && alpha <= 1.0)) return TMK_ERR_BAD_DESC;
  return fill(fine->coarser, alpha, (cudaStream_t)stream);
}

extern "C" tmk_status tmk_level_reflux(tmk_level* coarse, void* stream) {
  if (!coarse || !coarse->finer) return TMK_ERR_BAD_DESC;
  CFLink* k = coarse->finer;
  cudaStream_t s = (cudaStream_t)stream;
  return coarse->prec == TMK_PREC_MIXED ? launch_reflux<float>(k, s) : launch_reflux<double>(k, s);
}

extern "C" tmk_status tmk_level_average_down(tmk_level* coarse, void* stream) {
  if (!coarse || !coarse->finer) return TMK_ERR_BAD_DESC;
  CFLink* k = coarse->finer;
  cudaStream_t s = (cudaStream_t)stream;
  return coarse->prec == TMK_PREC_MIXED ? launch_avgdown<float>(k, s) : launch_avgdown<double>(k, s);
}

extern "C" tmk_status tmk_level_interp_from_coarser(tmk_level* fine, void* stream) {
  if (!fine || !fine->coarser) return TMK_ERR_BAD_DESC;
  CFLink* k = fine->coarser;
  cudaStream_t s = (cudaStream_t)stream;
  return fine->prec == TMK_PREC_MIXED ? launch_interp<float>(k, s) : launch_interp<double>(k, s);
}

extern "C" tmk_status tmk_level_copy_overlap(tmk_level* dst, const tmk_level* src, void* stream) {
  if (!dst || !src || dst == src || dst->prec != src->prec || dst->ctx->nb != src->ctx->nb) return TMK_ERR_BAD_DESC;
  if (dst->nscen != 1 || src->nscen != 1) return TMK_ERR_UNSUPPORTED;
  for (int d = 0; d < 2; ++d)
    if (dst->domain.lo[d] != src->domain.lo[d] || dst->domain.hi[d] != src->domain.hi[d]) return TMK_ERR_BAD_DESC;
  std::vector<CopyDev> cu, cb;
  for (size_t p = 0; p < dst->patches.size(); ++p)
    for (size_t q = 0; q < src->patches.size(); ++q) {
      const tmk_box x = box_isect(dst->patches[p].valid, src->patches[q].valid);
      if (!box_ok(x)) continue;
      CopyDev c; c.src = (int)q; c.dst = (int)p; c.lo0 = x.lo[0]; c.lo1 = x.lo[1]; c.hi0 = x.hi[0]; c.hi1 = x.hi[1];
      cu.push_back(c);
      if (dst->patches[p].fault && src->patches[q].fault && dst->ctx->nb > 0) { c.lo1 = c.hi1 = dst->domain.lo[1]; cb.push_back(c); }
    }
  if (cu.empty()) return TMK_OK;
  std::vector<CopyDev> all(cu);
  all.insert(all.end(), cb.begin(), cb.end());
  CopyDev* d = nullptr;
  if (dalloc(&d, all.size()) != cudaSuccess) return TMK_ERR_ALLOC;
  cudaStream_t s = (cudaStream_t)stream;
  tmk_status st = TMK_OK;
  if (cudaMemcpy(d, all.data(), all.size() * sizeof(CopyDev), cudaMemcpyHostToDevice) != cudaSuccess) st = TMK_ERR_CUDA;
  if (st == TMK_OK) {
    if (dst->prec == TMK_PREC_MIXED)
      xcopy_kernel<float><<<(unsigned)all.size(), 256, 0, s>>>((const PatchDev<float>*)dst->dpatch[dst->parity],
                                                               (const PatchDev<float>*)src->dpatch[src->parity], d,
                                                               (int)cu.size(), dst->ctx->nb);
    else
      xcopy_kernel<double><<<(unsigned)all.size(), 256, 0, s>>>((const PatchDev<double>*)dst->dpatch[dst->parity],
                                                                (const PatchDev<double>*)src->dpatch[src->parity], d,
                                                                (int)cu.size(), dst->ctx->nb);
    if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(s) != cudaSuccess) st = TMK_ERR_CUDA;
  }
  cudaFree(d);
  return st;
}

extern "C" tmk_status tmk_level_register_size(const tmk_level* fine, int* entries) {
  if (!fine || !entries || !fine->coarser) return TMK_ERR_BAD_DESC;
  *entries = fine->coarser->nent;
  return TMK_OK;
}

// --------------------------------------------------------------- hierarchy
struct tmk_amr_s {
  std::vector<tmk_level*> L;
  std::vector<int> ratio;
  std::vector<double> time, dtlast;
};

extern "C" tmk_status tmk_amr_create(int nlevels, tmk_level* const* levels, const int* ratios, double time,
                                     tmk_amr** out) {
  if (!out) return TMK_ERR_BAD_DESC;
  *out = nullptr;
  if (nlevels < 1 || !levels || (nlevels > 1 && !ratios)) return TMK_ERR_BAD_DESC;
  for (int l = 0; l < nlevels; ++l) if (!levels[l]) return TMK_ERR_BAD_DESC;
  if (levels[0]->coarser) detach(levels[0]);
  for (int l = 0; l + 1 < nlevels; ++l) {
    tmk_status st = tmk_level_attach_coarser(levels[l + 1], levels[l], ratios[l]);
    if (st != TMK_OK) return st;
  }
  if (levels[nlevels - 1]->finer) detach(levels[nlevels - 1]->finer->F);
  tmk_amr* h = new (std::nothrow) tmk_amr_s();
  if (!h) return TMK_ERR_ALLOC;
  h->L.assign(levels, levels + nlevels);
  if (nlevels > 1) h->ratio.assign(ratios, ratios + nlevels - 1);
  h->time.assign(nlevels, time);
  h->dtlast.assign(nlevels, 0.0);
  *out = h;
  return TMK_OK;
}

extern "C" void tmk_amr_destroy(tmk_amr* h) { delete h; }

namespace {
// AMR::timeStep: advance level l, then ratio[l] substeps of level l+1, then
// AMRLevelLinElast::postTimeStep (reflux, average-down of U and B)
tmk_status amr_advance(tmk_amr* h, int l, double dt, cudaStream_t s) {
  double tco = 0.0, tcn = 0.0;
  if (l > 0) { tcn = h->time[l - 1]; tco = tcn - h->dtlast[l - 1]; }
  tmk_status st = tmk_level_step_cf(h->L[l], h->time[l], dt, tco, tcn, s, nullptr);
  if (st != TMK_OK) return st;
  h->time[l] += dt;
  h->dtlast[l] = dt;
  if (l + 1 < (int)h->L.size()) {
    const int r = h->ratio[l];
    for (int k = 0; k < r; ++k)
      if ((st = amr_advance(h, l + 1, dt / r, s)) != TMK_OK) return st;
    if ((st = tmk_level_reflux(h->L[l], s)) != TMK_OK) return st;
    if ((st = tmk_level_average_down(h->L[l], s)) != TMK_OK) return st;
    if (h->L[l]->stations && (st = tmk_stations_record(h->L[l]->stations, h->time[l], s)) != TMK_OK) return st;
  }
  return TMK_OK;
}
}  // namespace

// Hierarchy autotuner: coordinate descent over the levels, finest first; each
// candidate tuning of a level is timed over whole subcycled coarse steps from
// the hierarchy's present state (put back before every trial and at the end).
extern "C" tmk_status tmk_amr_autotune(tmk_amr* h, double dt0, int ncoarse, void* stream, tmk_tuning* per_level,
                                       double* ms_per_coarse_step) {
  if (!h || !(dt0 > 0) || ncoarse < 1) return TMK_ERR_BAD_DESC;
  for (tmk_level* L : h->L) if (L->graphs || L->prof_on) return TMK_ERR_BAD_DESC;
  cudaStream_t s = (cudaStream_t)stream;
  TMK_CU(cudaDeviceSynchronize());
  const size_t nl = h->L.size();
  std::vector<LevelSnapshot> snaps(nl);
  for (size_t l = 0; l < nl; ++l) {
    tmk_status st = snaps[l].save(h->L[l]);
    if (st != TMK_OK) return st;
  }
  const std::vector<double> time0 = h->time, dtlast0 = h->dtlast;
  auto restore_all = [&]() -> tmk_status {
    for (size_t l = 0; l < nl; ++l) {
      tmk_status st = snaps[l].restore(h->L[l]);
      if (st != TMK_OK) return st;
    }
    h->time = time0;
    h->dtlast = dtlast0;
    return TMK_OK;
  };
  cudaEvent_t e0, e1;
  TMK_CU(cudaEventCreate(&e0));
  TMK_CU(cudaEventCreate(&e1));
  auto trial = [&](double* ms) -> tmk_status {
    tmk_status st = restore_all();
    if (st == TMK_OK) st = amr_advance(h, 0, dt0, s);
    if (st != TMK_OK) return st;
    TMK_CU(cudaEventRecord(e0, s));
    for (int k = 0; k < ncoarse; ++k)
      if ((st = amr_advance(h, 0, dt0, s)) != TMK_OK) return st;
    TMK_CU(cudaEventRecord(e1, s));
    TMK_CU(cudaEventSynchronize(e1));
    float f = 0.f;
    TMK_CU(cudaEventElapsedTime(&f, e0, e1));
    *ms = f / ncoarse;
    return TMK_OK;
  };
  tmk_status st = TMK_OK;
  double best_ms = 0.0;
  for (int l = (int)nl - 1; l >= 0 && st == TMK_OK; --l) {
    tmk_level_s* L = h->L[l];
    const tmk_tuning keep = L->tune;
    std::vector<tmk_tuning> cand = tuning_candidates(L, true);
    std::vector<std::pair<double, int>> timed;
    for (size_t k = 0; k < cand.size() && st == TMK_OK; ++k) {
      double ms = 0.0;
      if ((st = tmk_level_set_tuning(L, &cand[k])) != TMK_OK) break;
      if ((st = trial(&ms)) != TMK_OK) break;
      timed.push_back({ms, (int)k});
    }
    if (st != TMK_OK) { tmk_level_set_tuning(L, &keep); break; }
    std::sort(timed.begin(), timed.end());
    const size_t top = std::min<size_t>(3, timed.size());
    for (size_t r = 0; r < 2 && st == TMK_OK; ++r)
      for (size_t q = 0; q < top && st == TMK_OK; ++q) {
        double ms = 0.0;
        if ((st = tmk_level_set_tuning(L, &cand[timed[q].second])) != TMK_OK) break;
        if ((st = trial(&ms)) != TMK_OK) break;
        timed[q].first += ms;
      }
    size_t b = 0;
    for (size_t q = 1; q < top; ++q) if (timed[q].first < timed[b].first) b = q;
    const tmk_tuning pick = st == TMK_OK ? cand[timed[b].second] : keep;
    best_ms = timed[b].first / 3.0;
    tmk_status st2 = tmk_level_set_tuning(L, &pick);
    if (st == TMK_OK) st = st2;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  tmk_status st3 = restore_all();
  if (st == TMK_OK) st = st3;
  if (st == TMK_OK) {
    if (per_level) for (size_t l = 0; l < nl; ++l) per_level[l] = h->L[l]->tune;
    if (ms_per_coarse_step) *ms_per_coarse_step = best_ms;
  }
  return st;
}

extern "C" tmk_status tmk_amr_step(tmk_amr* h, double dt0, void* stream) {
  if (!h || !(dt0 > 0)) return TMK_ERR_BAD_DESC;
  return amr_advance(h, 0, dt0, (cudaStream_t)stream);
}

extern "C" tmk_status tmk_amr_time(const tmk_amr* h, int level, double* t) {
  if (!h || !t || level < 0 || level >= (int)h->L.size()) return TMK_ERR_BAD_DESC;
  *t = h->time[level];
  return TMK_OK;
}

extern "C" long long tmk_amr_cell_updates(const tmk_amr* h) {
  if (!h) return 0;
  long long total = 0, sub = 1;
  for (size_t l = 0; l < h->L.size(); ++l) {
    long long cells = 0;
    for (const LevelPatch& lp : h->L[l]->patches)
      cells += (long long)(lp.valid.hi[0] - lp.valid.lo[0] + 1) * (lp.valid.hi[1] - lp.valid.lo[1] + 1);
    total += cells * sub;
    if (l < h->ratio.size()) sub *= h->ratio[l];
  }
  return total;
}

extern "C" int tmk_amr_launches_per_step(const tmk_amr* h) {
  if (!h) return 0;
  int total = 0, sub = 1;
  for (size_t l = 0; l < h->L.size(); ++l) {
    int n = tmk_level_launches_per_step(h->L[l]);
    if (l + 1 < h->L.size()) {
      const CFLink* k = h->L[l]->finer;
      if (k && k->ncells) ++n;
      if (k && (k->nau || k->nab)) ++n;
    }
    total += n * sub;
    if (l < h->ratio.size()) sub *= h->ratio[l];
  }
  return total;
}

// ------------------------------------------------------------ CUDA graphs
// A captured sequence of level steps or AMR coarse steps.  Every step's
// launches are recorded once; a replay shifts the start-time argument of the
// captured fault-kernel nodes (the only launch argument that changes from one
// replay to the next) and launches the executable graph.
struct tmk_graph_s {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  std::vector<cudaGraphNode_t> tnodes;   // fault-kernel and station-kernel nodes
  std::vector<double> tbase;             // their time argument at capture
  std::vector<int> nparams;              // their parameter count
  double t0 = 0.0;                       // start time at capture
  double span = 0.0;                     // time advanced by one replay
  double dt0 = 0.0;                      // coarse step of an AMR graph
  tmk_amr* amr = nullptr;                // hierarchy whose host clock a replay advances
  std::vector<tmk_level_s*> levels;      // levels whose kernels the graph launches (their work
                                         // lists stay fixed while it exists)
};

namespace {

// parameter counts of fault_kernel and station_kernel
constexpr int kFaultParams = 5;
constexpr int kStationParams = 10;

tmk_status graph_finish(tmk_graph_s* g) {
  if (cudaGraphInstantiate(&g->exec, g->graph, 0) != cudaSuccess) return TMK_ERR_CUDA;
  size_t n = 0;
  if (cudaGraphGetNodes(g->graph, nullptr, &n) != cudaSuccess) return TMK_ERR_CUDA;
  std::vector<cudaGraphNode_t> nodes(n);
  if (n && cudaGraphGetNodes(g->graph, nodes.data(), &n) != cudaSuccess) return TMK_ERR_CUDA;
  // kernels whose fourth parameter is a time: the fault kernels (the step's
  // start) and the station kernels (the record's time)
  const void* fe[6] = {tmk::Launch<float>::fault_entry(tmk::FAULT_SEG),
                       tmk::Launch<float>::fault_entry(tmk::FAULT_SEG_SMALL),
                       tmk::Launch<double>::fault_entry(tmk::FAULT_SEG),
                       tmk::Launch<double>::fault_entry(tmk::FAULT_SEG_SMALL),
                       station_entry(TMK_PREC_MIXED), station_entry(TMK_PREC_FP64)};
  for (cudaGraphNode_t nd : nodes) {
    cudaGraphNodeType t;
    if (cudaGraphNodeGetType(nd, &t) != cudaSuccess) return TMK_ERR_CUDA;
    if (t != cudaGraphNodeTypeKernel) continue;
    cudaKernelNodeParams p;
    if (cudaGraphKernelNodeGetParams(nd, &p) != cudaSuccess) return TMK_ERR_CUDA;
    const int which = (int)(std::find(fe, fe + 6, p.func) - fe);
    if (which == 6) continue;
    g->tnodes.push_back(nd);
    g->tbase.push_back(*(const double*)p.kernelParams[3]);
    g->nparams.push_back(which < 4 ? kFaultParams : kStationParams);
  }
  return TMK_OK;
}

void graph_free(tmk_graph_s* g) {
  if (!g) return;
  for (tmk_level_s* L : g->levels) --L->graphs;
  if (g->exec) cudaGraphExecDestroy(g->exec);
  if (g->graph) cudaGraphDestroy(g->graph);
  delete g;
}

// descriptors of every level for its step size, before a capture (no host
// copies may happen while capturing)
tmk_status prepare_dt(tmk_level_s* L, double dt, cudaStream_t s) {
  if (dt == L->cur_dt) return TMK_OK;
  L->cur_dt = dt;
  if (upload_patchdev(L, s) != TMK_OK) return TMK_ERR_CUDA;
  TMK_CU(cudaStreamSynchronize(s));
  return TMK_OK;
}

}  // namespace

extern "C" tmk_status tmk_level_graph_create(tmk_level* L, int nsteps, double time, double dt, tmk_graph** out) {
  if (!out) return TMK_ERR_BAD_DESC;
  *out = nullptr;
  if (!L || nsteps <= 0 || (nsteps & 1) || !(dt > 0) || L->coarser || L->prof_on) return TMK_ERR_BAD_DESC;
  cudaStream_t cs;
  TMK_CU(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
  tmk_status st = prepare_dt(L, dt, cs);
  tmk_graph_s* g = st == TMK_OK ? new (std::nothrow) tmk_graph_s() : nullptr;
  if (st == TMK_OK && !g) st = TMK_ERR_ALLOC;
  if (st == TMK_OK && cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal) != cudaSuccess) st = TMK_ERR_CUDA;
  if (st == TMK_OK) {
    for (int k = 0; k < nsteps && st == TMK_OK; ++k) st = tmk_level_step(L, time + k * dt, dt, cs, nullptr);
    if (cudaStreamEndCapture(cs, &g->graph) != cudaSuccess && st == TMK_OK) st = TMK_ERR_CUDA;
  }
  if (st == TMK_OK) st = graph_finish(g);
  cudaStreamDestroy(cs);
  if (st != TMK_OK) { graph_free(g); return st; }
  g->t0 = time;
  g->span = nsteps * dt;
  g->levels.push_back(L);
  ++L->graphs;
  *out = g;
  return TMK_OK;
}

extern "C" tmk_status tmk_amr_graph_create(tmk_amr* h, int ncoarse, double dt0, tmk_graph** out) {
  if (!out) return TMK_ERR_BAD_DESC;
  *out = nullptr;
  if (!h || ncoarse <= 0 || (ncoarse & 1) || !(dt0 > 0)) return TMK_ERR_BAD_DESC;
  for (tmk_level* L : h->L) if (L->prof_on) return TMK_ERR_BAD_DESC;
  cudaStream_t cs;
  TMK_CU(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
  tmk_status st = TMK_OK;
  double dtl = dt0;
  for (size_t l = 0; l < h->L.size() && st == TMK_OK; ++l) {
    st = prepare_dt(h->L[l], dtl, cs);
    if (l < h->ratio.size()) dtl /= h->ratio[l];
  }
  const std::vector<double> time0 = h->time, dtlast0 = h->dtlast;
  tmk_graph_s* g = st == TMK_OK ? new (std::nothrow) tmk_graph_s() : nullptr;
  if (st == TMK_OK && !g) st = TMK_ERR_ALLOC;
  if (st == TMK_OK && cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal) != cudaSuccess) st = TMK_ERR_CUDA;
  if (st == TMK_OK) {
    for (int k = 0; k < ncoarse && st == TMK_OK; ++k) st = amr_advance(h, 0, dt0, cs);
    if (cudaStreamEndCapture(cs, &g->graph) != cudaSuccess && st == TMK_OK) st = TMK_ERR_CUDA;
  }
  // nothing ran: the hierarchy's clock stays where it was
  h->time = time0;
  h->dtlast = dtlast0;
  if (st == TMK_OK) st = graph_finish(g);
  cudaStreamDestroy(cs);
  if (st != TMK_OK) { graph_free(g); return st; }
  g->t0 = time0[0];
  g->span = ncoarse * dt0;
  g->dt0 = dt0;
  g->amr = h;
  for (tmk_level* L : h->L) { g->levels.push_back(L); ++L->graphs; }
  *out = g;
  return TMK_OK;
}

extern "C" tmk_status tmk_graph_launch(tmk_graph* g, double time, void* stream) {
  if (!g || !g->exec) return TMK_ERR_BAD_DESC;
  const double shift = time - g->t0;
  for (size_t k = 0; k < g->tnodes.size(); ++k) {
    cudaKernelNodeParams p;
    TMK_CU(cudaGraphKernelNodeGetParams(g->tnodes[k], &p));
    double t = g->tbase[k] + shift;
    void* args[kStationParams];
    for (int q = 0; q < g->nparams[k]; ++q) args[q] = p.kernelParams[q];
    args[3] = &t;
    p.kernelParams = args;
    TMK_CU(cudaGraphExecKernelNodeSetParams(g->exec, g->tnodes[k], &p));
  }
  TMK_CU(cudaGraphLaunch(g->exec, (cudaStream_t)stream));
  if (g->amr) {   // the hierarchy's clock after the replayed coarse steps
    tmk_amr* h = g->amr;
    double dtl = g->dt0;
    for (size_t l = 0; l < h->L.size(); ++l) {
      h->time[l] = time + g->span;
      h->dtlast[l] = dtl;
      if (l < h->ratio.size()) dtl /= h->ratio[l];
    }
  }
  return TMK_OK;
}

extern "C" void tmk_graph_destroy(tmk_graph* g) { graph_free(g); }
