// tmk_regrid.cu -- refinement tagging on the device.
//
// AMRLevelLinElast::tagCells / tagCellsInit (srcLinElast/AMRLevelLinElast.cpp:
// 577-717, 721-771): per valid cell of every patch, the largest undivided
// difference of side 1's velocities (GETFULLGRADF + MAXF,
// srcLinElast/LinElastPhysicsF.ChF:59-82, 199-259), the fault law's nucleation
// marks (RSIBC/SWIBC::tagCellsInit), the coarsening-scaled threshold, the
// coarsen2 window and the plastic-strain test; then IntVectSet::grow by the
// tag buffer as two separable max filters over a byte mask of the domain.
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
      tag = window && (gm >= thr || uat(p, 10, i, j) >= tc.pthr || uat(p, 21, i, j) >= tc.pthr);
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
