// tmk_launch_impl.cuh -- bodies of the launch wrappers; included by exactly one
// translation unit per arithmetic type.
#pragma once
#include "tmk_kernels.cuh"
#include "tmk_march.cuh"
#include "tmk_launch.h"

namespace tmk {

template <typename Real, int TX_, int TY_, int NT_>
struct LaunchImpl {
  static cudaError_t fault(const PatchDev<Real>* patches, const int* fp, int nfault, int max_faces,
                           const DevParams* params, double time, DevStatus* st, cudaStream_t s) {
    if (nfault <= 0) return cudaSuccess;
    dim3 grid((max_faces + 2 + 127) / 128, nfault);
    fault_kernel<Real><<<grid, 128, 0, s>>>(patches, fp, params, time, st);
    return cudaGetLastError();
  }
  static size_t smem() { return sizeof(VolSmem<Real, TX_, TY_>); }
  static cudaError_t volume(const PatchDev<Real>* patches, const TileDev* tiles, int ntiles,
                            const DevParams* params, cudaStream_t s) {
    if (ntiles <= 0) return cudaSuccess;
    static bool configured = false;
    const size_t sm = smem();
    if (!configured) {
      cudaError_t e = cudaFuncSetAttribute(volume_kernel<Real, TX_, TY_, NT_>,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
      if (e != cudaSuccess) return e;
      configured = true;
    }
    dim3 grid(ntiles, 2);
    volume_kernel<Real, TX_, TY_, NT_><<<grid, NT_, sm, s>>>(patches, tiles, params);
    return cudaGetLastError();
  }
  static cudaError_t exchange(const PatchDev<Real>* patches, const CopyDev* copies, int ncopies, int c0,
                              int ncomp, cudaStream_t s) {
    if (ncopies <= 0) return cudaSuccess;
    exchange_kernel<Real><<<ncopies, 256, 0, s>>>(patches, copies, c0, ncomp, 0);
    return cudaGetLastError();
  }
  static cudaError_t march(const PatchDev<Real>* patches, const MarchItem* items, int nitems,
                           const DevParams* params, cudaStream_t s) {
    if (nitems <= 0) return cudaSuccess;
    const int blocks = (nitems + MARCH_WARPS - 1) / MARCH_WARPS;
    march_kernel<Real, 0><<<blocks, 32 * MARCH_WARPS, 0, s>>>(patches, items, nitems, params);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    march_kernel<Real, 1><<<blocks, 32 * MARCH_WARPS, 0, s>>>(patches, items, nitems, params);
    return cudaGetLastError();
  }
};

}  // namespace tmk

#define TMK_INSTANTIATE_LAUNCH(REAL, TXV, TYV, NTV)                                                          \
  namespace tmk {                                                                                            \
  template <> const int Launch<REAL>::TX = TXV;                                                             \
  template <> const int Launch<REAL>::TY = TYV;                                                             \
  template <> cudaError_t Launch<REAL>::fault(const PatchDev<REAL>* p, const int* fp, int nf, int mf,        \
                                              const DevParams* prm, double t, DevStatus* st, cudaStream_t s) { \
    return LaunchImpl<REAL, TXV, TYV, NTV>::fault(p, fp, nf, mf, prm, t, st, s);                             \
  }                                                                                                          \
  template <> cudaError_t Launch<REAL>::volume(const PatchDev<REAL>* p, const TileDev* tl, int nt,          \
                                               const DevParams* prm, cudaStream_t s) {                      \
    return LaunchImpl<REAL, TXV, TYV, NTV>::volume(p, tl, nt, prm, s);                                       \
  }                                                                                                          \
  template <> cudaError_t Launch<REAL>::exchange(const PatchDev<REAL>* p, const CopyDev* c, int n, int c0,  \
                                                 int nc, cudaStream_t s) {                                   \
    return LaunchImpl<REAL, TXV, TYV, NTV>::exchange(p, c, n, c0, nc, s);                                    \
  }                                                                                                          \
  template <> size_t Launch<REAL>::volume_smem() { return LaunchImpl<REAL, TXV, TYV, NTV>::smem(); }         \
  template <> cudaError_t Launch<REAL>::march(const PatchDev<REAL>* p, const MarchItem* it, int n,           \
                                              const DevParams* prm, cudaStream_t s) {                       \
    return LaunchImpl<REAL, TXV, TYV, NTV>::march(p, it, n, prm, s);                                         \
  }                                                                                                          \
  }
