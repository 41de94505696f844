// tmk_regrid.cu -- refinement tagging on the device.
//
// AMRLevelLinElast::tagCells / tagCellsInit (srcLinElast/AMRLevelLinElast.cpp:
// 577-717, 721-771): per valid cell of every patch, the largest undivided
// difference of side 1's velocities (GETFULLGRADF + MAXF,
// srcLinElast/LinElastPhysicsF.ChF:59-82, 199-259), the fault law's nucleation
// marks (RSIBC/SWIBC::tagCellsInit), the coarsening-scaled threshold, the
// coarsen2 window and the plastic-strain test (plus, as an extension, a
// slip-rate test on the fault row); then IntVectSet::grow by the tag buffer as
// two separable max filters over a byte mask of the domain.
// Built with --fmad=false: the FP64 form tags exactly as the oracle does.
#include <cmath>
#include <cstring>
#include "tmk_internal.h"

using namespace tmk;
using namespace tmk_host;

namespace {

constexpr int kMaxNuc = TMK_SW_MAX_PATCHES;

struct TagConst {
  double dx, thr, pthr, xc0, xc1, yc0, yc1, slope, width, x20, x21, y20, y21;
  double vthr;           // slip-rate threshold of the fault-row tag (<= 0: off)
  int vcomp;             // the slip-rate component of the boundary data
  int window_always;     // level < coarsen2_max_level
  int initial, marks;    // tagCellsInit; the fault law marks nucleation cells
  int nnuc;
  int nlo[kMaxNuc], nhi[kMaxNuc];   // nucleation x ranges on row j = 0
  int dlo0, dlo1, dhi0, dhi1;
};

template <typename Real>
__device__ __forceinline__ double uat(const PatchDev<Real>& p, int c, int i, int j) {
  return (double)p.Uin[fab_idx(p, c, i, j)];
}

template <typename Real>
__global__ void tag_kernel(const PatchDev<Real>* __restrict__ patches, const TagConst tc,
                           unsigned char* __restrict__ raw) {
  const PatchDev<Real>& p = patches[blockIdx.y];
  const int nvx = p.vhi0 - p.vlo0 + 1, nvy = p.vhi1 - p.vlo1 + 1;
  const int mnx = tc.dhi0 - tc.dlo0 + 1;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nvx * nvy; t += gridDim.x * blockDim.x) {
    const int i = p.vlo0 + t % nvx, j = p.vlo1 + t / nvx;
    bool nuc = false;
    if (j == 0)
      for (int k = 0; k < tc.nnuc; ++k)
        if (i >= tc.nlo[k] && i <= tc.nhi[k]) nuc = true;
    bool tag;
    if (tc.initial) {
      tag = tc.marks && nuc;
    } else {
      double grad[2];
#pragma unroll
      for (int d = 0; d < 2; ++d) {
        const int e0 = d == 0, e1 = d == 1, k = d == 0 ? i : j;
        const int lo = d == 0 ? tc.dlo0 : tc.dlo1, hi = d == 0 ? tc.dhi0 : tc.dhi1;
        double diff = 0.0;
        for (int iv = 0; iv <= 2; ++iv) {
          double v;
          if (k > lo && k < hi) v = 0.5 * fabs(uat(p, iv, i + e0, j + e1) - uat(p, iv, i - e0, j - e1));
          else if (k == lo) v = fabs(uat(p, iv, i + e0, j + e1) - uat(p, iv, i, j));
          else v = fabs(uat(p, iv, i, j) - uat(p, iv, i - e0, j - e1));
          diff = (diff < v) ? v : diff;
        }
        grad[d] = diff;
      }
      double gm = 0.0;
      for (int d = 0; d < 2; ++d) { const double a = fabs(grad[d]); gm = (gm < a) ? a : gm; }
      if (nuc) gm = 1.0;
      const double x = i * tc.dx, y = j * tc.dx;
      double r = 0;
      { const double a = tc.xc0 - x, b = x - tc.xc1; const double m = (a < b) ? b : a; r = (r < m) ? m : r; }
      { const double a = tc.yc0 - y, b = y - tc.yc1; const double m = (a < b) ? b : a; r = (r < m) ? m : r; }
      const double thr = tc.thr * (1 + r * tc.slope / tc.width);
      const bool window = tc.window_always || (x >= tc.x20 && x <= tc.x21 && y >= tc.y20 && y <= tc.y21);
      // slip-rate tag of the fault row (an extension): the slip rate of the face below the cell
      const bool slip = tc.vthr > 0 && p.fault && j == tc.dlo1 &&
                        p.B[(size_t)tc.vcomp * p.bnx + (i - p.blo0)] >= tc.vthr;
      tag = window && (gm >= thr || uat(p, 10, i, j) >= tc.pthr || uat(p, 21, i, j) >= tc.pthr || slip);
    }
    if (tag) raw[(size_t)(j - tc.dlo1) * mnx + (i - tc.dlo0)] = 1;
  }
}

// one pass of IntVectSet::grow(n): the max over a window of 2n+1 cells along x (dir 0) or y
__global__ void dilate_kernel(const unsigned char* __restrict__ in, unsigned char* __restrict__ out, int nx, int ny,
                              int n, int dir) {
  const long long total = (long long)nx * ny;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(t % nx), j = (int)(t / nx);
    unsigned char v = 0;
    if (dir == 0) {
      for (int ii = max(0, i - n); ii <= min(nx - 1, i + n); ++ii) v |= in[(size_t)j * nx + ii];
    } else {
      for (int jj = max(0, j - n); jj <= min(ny - 1, j + n); ++jj) v |= in[(size_t)jj * nx + i];
    }
    out[t] = v;
  }
}

template <typename Real>
tmk_status tag_launch(tmk_level_s* L, const TagConst& tc, unsigned char* raw, cudaStream_t s) {
  int maxc = 1;
  for (const LevelPatch& lp : L->patches)
    maxc = std::max(maxc, (lp.valid.hi[0] - lp.valid.lo[0] + 1) * (lp.valid.hi[1] - lp.valid.lo[1] + 1));
  const PatchDev<Real>* pd = (const PatchDev<Real>*)L->dpatch[L->parity];
  if (!tc.initial) TMK_CU(Launch<Real>::exchange(pd, L->dcopies, L->ncopies, 0, TMK_NCOMP, s));
  dim3 grid(std::min(64, (maxc + 255) / 256), (unsigned)L->patches.size());
  tag_kernel<Real><<<grid, 256, 0, s>>>(pd, tc, raw);
  TMK_CU(cudaGetLastError());
  return TMK_OK;
}

}  // namespace

extern "C" tmk_status tmk_level_tag_cells(tmk_level* L, const tmk_tag_params* tp, unsigned char* mask, int host,
                                          void* stream) {
  if (!L || !tp || !mask || tp->tag_buffer < 0) return TMK_ERR_BAD_DESC;
  if (L->nscen != 1) return TMK_ERR_UNSUPPORTED;
  cudaStream_t s = (cudaStream_t)stream;
  const DevParams& P = L->ctx->hp;
  TagConst tc;
  std::memset(&tc, 0, sizeof(tc));
  tc.dx = L->dx; tc.thr = tp->refine_thresh; tc.pthr = tp->plastic_thresh;
  tc.xc0 = tp->x_coarsen[0]; tc.xc1 = tp->x_coarsen[1]; tc.yc0 = tp->y_coarsen[0]; tc.yc1 = tp->y_coarsen[1];
  tc.slope = tp->slope_coarsen; tc.width = tp->width_coarsen;
  tc.x20 = tp->x_coarsen2[0]; tc.x21 = tp->x_coarsen2[1]; tc.y20 = tp->y_coarsen2[0]; tc.y21 = tp->y_coarsen2[1];
  tc.window_always = tp->level < tp->coarsen2_max_level ? 1 : 0;
  tc.initial = tp->initial ? 1 : 0;
  tc.vthr = P.fault_law == 0 ? 0.0 : tp->slip_rate_thresh;
  tc.vcomp = P.fault_law == 2 ? 4 : 2;     // RSSETBND V / SWSETBND V
  tc.dlo0 = L->domain.lo[0]; tc.dlo1 = L->domain.lo[1]; tc.dhi0 = L->domain.hi[0]; tc.dhi1 = L->domain.hi[1];
  // RSIBC::tagCellsInit (ibcLinElast/RSIBC.cpp:351-368) / SWIBC::tagCellsInit (ibcLinElast/SWIBC.cpp:340-372)
  if (P.fault_law == 1) {
    tc.marks = 1; tc.nnuc = 1;
    tc.nlo[0] = (int)std::floor(P.rs_x0 / L->dx);
    tc.nhi[0] = (int)std::ceil(P.rs_x0 / L->dx);
  } else if (P.fault_law == 2) {
    tc.marks = 1; tc.nnuc = std::min(P.sw_np, kMaxNuc);
    for (int k = 0; k < tc.nnuc; ++k) {
      tc.nlo[k] = (int)std::floor((P.sw_fbc0 + P.sw_xc[k] - P.sw_xw[k]) / L->dx);
      tc.nhi[k] = (int)std::ceil((P.sw_fbc0 + P.sw_xc[k] + P.sw_xw[k]) / L->dx);
    }
  }
  // ghost cells as the reference fills them before tagging: from the coarser
  // level's new state (alpha = 1), then by exchange (in tag_launch)
  if (!tp->initial && L->coarser) {
    tmk_status st = tmk_level_fill_coarse_fine(L, 1.0, stream);
    if (st != TMK_OK) return st;
  }
  const int nx = L->domain.hi[0] - L->domain.lo[0] + 1, ny = L->domain.hi[1] - L->domain.lo[1] + 1;
  const size_t n = (size_t)nx * ny;
  unsigned char* buf = nullptr;
  TMK_CU(cudaMalloc(&buf, 3 * n));
  unsigned char *raw = buf, *tmp = buf + n, *out = host ? buf + 2 * n : mask;
  tmk_status st = TMK_OK;
  if (cudaMemsetAsync(raw, 0, n, s) != cudaSuccess) st = TMK_ERR_CUDA;
  if (st == TMK_OK)
    st = L->prec == TMK_PREC_MIXED ? tag_launch<float>(L, tc, raw, s) : tag_launch<double>(L, tc, raw, s);
  if (st == TMK_OK) {
    const int blocks = (int)std::min<long long>(4096, ((long long)n + 255) / 256);
    dilate_kernel<<<blocks, 256, 0, s>>>(raw, tmp, nx, ny, tp->tag_buffer, 0);
    dilate_kernel<<<blocks, 256, 0, s>>>(tmp, out, nx, ny, tp->tag_buffer, 1);
    if (cudaGetLastError() != cudaSuccess) st = TMK_ERR_CUDA;
  }
  if (st == TMK_OK && host && cudaMemcpyAsync(mask, out, n, cudaMemcpyDeviceToHost, s) != cudaSuccess) st = TMK_ERR_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess && st == TMK_OK) st = TMK_ERR_CUDA;
  cudaFree(buf);
  return st;
}

// ================================================================ stations
// AMRLevelLinElast::writeStationLevel (srcLinElast/AMRLevelLinElast.cpp:1758-1869)
// with the station cells and weights of AMRLevelLinElast::define (:257-335).
// Each record is one launch of one CTA: the record slot is taken from a
// device counter, so recording is asynchronous and can sit in a CUDA graph.
namespace {

struct StationDev {
  int kind;            // 0 fault (B, nb values), 1 body (U, 22 values)
  int off;             // first value of the station in a record (after the time)
  int present;         // a patch of the level holds the station's cell
  int p[4], i[4], j[4];  // the interpolation's cells: owning patch (or the station patch's ghost) and index
  double wx, wy;       // the reference's weights (distances from the cell centre, not divided by dx)
};

template <typename Real>
__global__ void station_kernel(const StationDev* __restrict__ st, int n, const PatchDev<Real>* __restrict__ patches,
                               double time, double* __restrict__ rec, int* __restrict__ count,
                               unsigned long long* __restrict__ dropped, int capacity, int stride, int nb) {
  __shared__ int slot;
  if (threadIdx.x == 0) {
    const int k = *count;
    slot = k;
    if (k < capacity) *count = k + 1;
    else *dropped += 1ull;
  }
  __syncthreads();
  if (slot >= capacity) return;
  double* r = rec + (size_t)slot * stride;
  if (threadIdx.x == 0) r[0] = time;
  for (int s = 0; s < n; ++s) {
    const StationDev& d = st[s];
    const int nv = d.kind == 0 ? nb : NC;
    for (int c = threadIdx.x; c < nv; c += blockDim.x) {
      double v;
      if (!d.present) {
        v = __longlong_as_double(0x7ff8000000000000ll);   // NaN: no patch of this level holds it
      } else if (d.kind == 0) {
        const PatchDev<Real>& p0 = patches[d.p[0]];
        const PatchDev<Real>& p1 = patches[d.p[1]];
        const double b0 = p0.B[(size_t)c * p0.bnx + (d.i[0] - p0.blo0)];
        const double b1 = p1.B[(size_t)c * p1.bnx + (d.i[1] - p1.blo0)];
        v = b0 * (1 - d.wx) + b1 * d.wx;
      } else {
        double u[4];
        for (int k = 0; k < 4; ++k) {
          const PatchDev<Real>& pk = patches[d.p[k]];
          u[k] = (double)pk.Uin[fab_idx(pk, c, d.i[k], d.j[k])];
        }
        v = u[0] * (1 - d.wx) * (1 - d.wy) + u[1] * d.wx * (1 - d.wy) + u[2] * (1 - d.wx) * d.wy +
            u[3] * d.wx * d.wy;
      }
      r[1 + d.off + c] = v;
    }
  }
}

}  // namespace

struct tmk_stations_s {
  tmk_level_s* L = nullptr;
  std::vector<StationDev> h;
  StationDev* d = nullptr;
  double* rec = nullptr;
  int* count = nullptr;
  unsigned long long* dropped = nullptr;
  int capacity = 0, stride = 1;
};

const void* tmk_host::station_entry(int prec) {
  return prec == TMK_PREC_MIXED ? (const void*)station_kernel<float> : (const void*)station_kernel<double>;
}

namespace {

// patch whose valid box holds cell (i, j), else -1
int owner(const tmk_level_s* L, int i, int j) {
  for (size_t p = 0; p < L->patches.size(); ++p) {
    const tmk_box& v = L->patches[p].valid;
    if (i >= v.lo[0] && i <= v.hi[0] && j >= v.lo[1] && j <= v.hi[1]) return (int)p;
  }
  return -1;
}

}  // namespace

extern "C" tmk_status tmk_stations_create(tmk_level* L, int nfault, const double* x_fault, int nbody,
                                          const double* x_body, const double* y_body, const double* center,
                                          int capacity, tmk_stations** out) {
  if (!out) return TMK_ERR_BAD_DESC;
  *out = nullptr;
  if (!L || nfault < 0 || nbody < 0 || nfault + nbody == 0 || capacity < 1 || !center) return TMK_ERR_BAD_DESC;
  if ((nfault && !x_fault) || (nbody && (!x_body || !y_body))) return TMK_ERR_BAD_DESC;
  if (L->nscen != 1) return TMK_ERR_UNSUPPORTED;
  if (nfault && L->ctx->nb == 0) return TMK_ERR_BAD_DESC;
  const double dx = L->dx;
  const int nb = L->ctx->nb;
  const int jf = L->domain.lo[1];
  tmk_stations_s* S = new (std::nothrow) tmk_stations_s();
  if (!S) return TMK_ERR_ALLOC;
  S->L = L;
  int off = 0;
  for (int k = 0; k < nfault + nbody; ++k) {
    StationDev s;
    std::memset(&s, 0, sizeof(s));
    const bool fault = k < nfault;
    s.kind = fault ? 0 : 1;
    s.off = off;
    off += fault ? nb : TMK_NCOMP;
    // AMRLevelLinElast::define (:260-335): the cell below the station and the
    // distances to its centre (in 2-D the z terms vanish)
    const double x = fault ? x_fault[k] : x_body[k - nfault];
    const int i0 = (int)std::floor((x + center[0]) / dx - 0.5);
    s.wx = -(i0 + 0.5) * dx + (x + center[0]);
    int j0 = jf;
    if (!fault) {
      const double y = y_body[k - nfault];
      j0 = (int)std::floor((y + center[1]) / dx - 0.5);
      s.wy = -(j0 + 0.5) * dx + (y + center[1]);
    }
    if (fault) {
      // the fault row of a patch holding face i0 (the reference's m_bdryGrids)
      int p0 = -1;
      for (size_t p = 0; p < L->patches.size(); ++p) {
        const LevelPatch& lp = L->patches[p];
        if (lp.fault && i0 >= lp.valid.lo[0] && i0 <= lp.valid.hi[0]) p0 = (int)p;
      }
      s.present = p0 >= 0;
      if (s.present) {
        int p1 = -1;
        for (size_t p = 0; p < L->patches.size(); ++p) {
          const LevelPatch& lp = L->patches[p];
          if (lp.fault && i0 + 1 >= lp.valid.lo[0] && i0 + 1 <= lp.valid.hi[0]) p1 = (int)p;
        }
        s.p[0] = p0; s.i[0] = i0;
        s.p[1] = p1 >= 0 ? p1 : p0; s.i[1] = i0 + 1;   // else the station patch's ghost face
      }
    } else {
      const int p0 = owner(L, i0, j0);
      s.present = p0 >= 0;
      if (s.present)
        for (int q = 0; q < 4; ++q) {
          const int ii = i0 + (q & 1), jj = j0 + (q >> 1);
          const int pq = owner(L, ii, jj);
          s.p[q] = pq >= 0 ? pq : p0;                  // else the station patch's ghost cell
          s.i[q] = ii; s.j[q] = jj;
        }
    }
    S->h.push_back(s);
  }
  S->stride = 1 + off;
  S->capacity = capacity;
  const size_t recb = (size_t)capacity * S->stride * sizeof(double);
  if (dalloc(&S->d, S->h.size()) != cudaSuccess || cudaMalloc(&S->rec, recb) != cudaSuccess ||
      dalloc(&S->count, 1) != cudaSuccess || dalloc(&S->dropped, 1) != cudaSuccess) {
    tmk_stations_destroy(S);
    return TMK_ERR_ALLOC;
  }
  if (cudaMemcpy(S->d, S->h.data(), S->h.size() * sizeof(StationDev), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemset(S->count, 0, sizeof(int)) != cudaSuccess ||
      cudaMemset(S->dropped, 0, sizeof(unsigned long long)) != cudaSuccess) {
    tmk_stations_destroy(S);
    return TMK_ERR_CUDA;
  }
  *out = S;
  return TMK_OK;
}

extern "C" void tmk_stations_destroy(tmk_stations* S) {
  if (!S) return;
  cudaDeviceSynchronize();
  if (S->L && S->L->stations == S) S->L->stations = nullptr;
  cudaFree(S->d); cudaFree(S->rec); cudaFree(S->count); cudaFree(S->dropped);
  delete S;
}

extern "C" tmk_status tmk_stations_record(tmk_stations* S, double time, void* stream) {
  if (!S || !S->L) return TMK_ERR_BAD_DESC;
  tmk_level_s* L = S->L;
  cudaStream_t s = (cudaStream_t)stream;
  const int n = (int)S->h.size(), nb = L->ctx->nb;
  if (L->prec == TMK_PREC_MIXED)
    station_kernel<float><<<1, 64, 0, s>>>(S->d, n, (const PatchDev<float>*)L->dpatch[L->parity], time, S->rec,
                                           S->count, S->dropped, S->capacity, S->stride, nb);
  else
    station_kernel<double><<<1, 64, 0, s>>>(S->d, n, (const PatchDev<double>*)L->dpatch[L->parity], time, S->rec,
                                            S->count, S->dropped, S->capacity, S->stride, nb);
  TMK_CU(cudaGetLastError());
  return TMK_OK;
}

extern "C" tmk_status tmk_stations_layout(const tmk_stations* S, int* values_per_record, int* present) {
  if (!S) return TMK_ERR_BAD_DESC;
  if (values_per_record) *values_per_record = S->stride;
  if (present)
    for (size_t k = 0; k < S->h.size(); ++k) present[k] = S->h[k].present;
  return TMK_OK;
}

extern "C" tmk_status tmk_stations_read(tmk_stations* S, double* out, int max_records, int* nrec,
                                        long long* dropped) {
  if (!S || !nrec || (max_records > 0 && !out)) return TMK_ERR_BAD_DESC;
  TMK_CU(cudaDeviceSynchronize());
  int n = 0;
  unsigned long long dr = 0;
  TMK_CU(cudaMemcpy(&n, S->count, sizeof(int), cudaMemcpyDeviceToHost));
  TMK_CU(cudaMemcpy(&dr, S->dropped, sizeof(dr), cudaMemcpyDeviceToHost));
  const int take = std::min(n, std::max(0, max_records));
  if (take) TMK_CU(cudaMemcpy(out, S->rec, (size_t)take * S->stride * sizeof(double), cudaMemcpyDeviceToHost));
  // records beyond max_records are dropped with the rest at the reset
  dr += (unsigned long long)(n - take);
  TMK_CU(cudaMemset(S->count, 0, sizeof(int)));
  TMK_CU(cudaMemset(S->dropped, 0, sizeof(unsigned long long)));
  *nrec = take;
  if (dropped) *dropped = (long long)dr;
  return TMK_OK;
}

extern "C" tmk_status tmk_level_attach_stations(tmk_level* L, tmk_stations* S) {
  if (!L || (S && S->L != L) || L->graphs) return TMK_ERR_BAD_DESC;
  L->stations = S;
  return TMK_OK;
}
