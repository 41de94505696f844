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
                           const DevParams* params, double time, DevStatus* st, bool pdl, int seg,
                           cudaStream_t s) {
    if (nfault <= 0) return cudaSuccess;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t cfg = {};
    const bool small = seg == FAULT_SEG_SMALL;
    const int sg = small ? FAULT_SEG_SMALL : FAULT_SEG;
    cfg.gridDim = dim3((max_faces + sg - 1) / sg, nfault);
    cfg.blockDim = dim3(small ? FAULT_THREADS_SMALL : FAULT_THREADS);
    cfg.stream = s;
    cfg.attrs = pdl ? attr : nullptr;
    cfg.numAttrs = pdl ? 1 : 0;
    if (small)
      return cudaLaunchKernelEx(&cfg, fault_kernel<Real, FAULT_SEG_SMALL, FAULT_THREADS_SMALL>, patches, fp,
                                params, time, st);
    return cudaLaunchKernelEx(&cfg, fault_kernel<Real, FAULT_SEG, FAULT_THREADS>, patches, fp, params, time, st);
  }
  static size_t smem() { return sizeof(VolSmem<Real, TX_, TY_>); }
  static int box_x() { return VolSmem<Real, TX_, TY_>::RXP; }
  static int box_y() { return VolSmem<Real, TX_, TY_>::RY; }
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
  static cudaError_t plastic(const PatchDev<Real>* patches, const TileDev* tiles, int ntiles,
                             const DevParams* params, cudaStream_t s) {
    if (ntiles <= 0) return cudaSuccess;
    plastic_tiles_kernel<Real><<<ntiles, 256, 0, s>>>(patches, tiles, params);
    return cudaGetLastError();
  }
  static cudaError_t exchange(const PatchDev<Real>* patches, const CopyDev* copies, int ncopies, int c0,
                              int ncomp, cudaStream_t s) {
    if (ncopies <= 0) return cudaSuccess;
    // about two waves of 256-thread CTAs: each copy box spread over up to 8 CTAs
    const int chunks = std::max(1, std::min(8, (2 * 8 * 152 + ncopies - 1) / ncopies));
    exchange_kernel<Real><<<dim3(ncopies, chunks), 256, 0, s>>>(patches, copies, c0, ncomp, 0);
    return cudaGetLastError();
  }
  static cudaError_t march(int g, const PatchDev<Real>* patches, const MarchItem* items, int nitems,
                           const MarchConst<Real>& mc, bool pdl, cudaStream_t s) {
    if (nitems <= 0) return cudaSuccess;
    static bool configured = false;
    if (!configured) {
      cudaError_t e = march_configure<MARCH_SCH_RUNTIME>();
      if (e == cudaSuccess) e = march_configure<MARCH_SCH_PPM_PRIM>();
      if (e != cudaSuccess) return e;
      configured = true;
    }
    const bool fx = march_scheme_fixed(mc);
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.blockDim = dim3(32 * MARCH_WARPS);
    cfg.gridDim = dim3((nitems + MARCH_WARPS - 1) / MARCH_WARPS);
    cfg.stream = s;
    cfg.attrs = pdl ? attr : nullptr;
    cfg.numAttrs = pdl ? 1 : 0;
    if (g == 0) {
      cfg.dynamicSmemBytes = march_smem_bytes<Real, 0>();
      if (mc.plastic)
        return fx ? cudaLaunchKernelEx(&cfg, march_kernel<Real, 0, true, MARCH_SCH_PPM_PRIM>, patches, items, nitems, mc)
                  : cudaLaunchKernelEx(&cfg, march_kernel<Real, 0, true>, patches, items, nitems, mc);
      return fx ? cudaLaunchKernelEx(&cfg, march_kernel<Real, 0, false, MARCH_SCH_PPM_PRIM>, patches, items, nitems, mc)
                : cudaLaunchKernelEx(&cfg, march_kernel<Real, 0>, patches, items, nitems, mc);
    }
    cfg.dynamicSmemBytes = march_smem_bytes<Real, 1>();
    return fx ? cudaLaunchKernelEx(&cfg, march_kernel<Real, 1, false, MARCH_SCH_PPM_PRIM>, patches, items, nitems, mc)
              : cudaLaunchKernelEx(&cfg, march_kernel<Real, 1>, patches, items, nitems, mc);
  }
  // the dynamic shared memory limit of the marching kernels of one scheme form
  template <int SCH>
  static cudaError_t march_configure() {
    cudaError_t e = cudaFuncSetAttribute(march_kernel<Real, 0, false, SCH>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)march_smem_bytes<Real, 0>());
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(march_kernel<Real, 1, false, SCH>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)march_smem_bytes<Real, 1>());
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(march_kernel<Real, 0, true, SCH>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)march_smem_bytes<Real, 0>());
    return e;
  }
  template <int G, bool PL, int SCH>
  static int march_blocks() {
    int b = 0;
    cudaFuncSetAttribute(march_kernel<Real, G, PL, SCH>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)march_smem_bytes<Real, G>());
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, march_kernel<Real, G, PL, SCH>, 32 * MARCH_WARPS,
                                                      march_smem_bytes<Real, G>()) != cudaSuccess)
      return 0;
    return b;
  }
  static cudaError_t march_fault_rows(const PatchDev<Real>* patches, const MarchItem* rows0, int n0,
                                      const MarchItem* rows1, int n1, const MarchConst<Real>& mc, cudaStream_t s) {
    if (n0 + n1 <= 0) return cudaSuccess;
    const int blocks = (n0 + n1 + MARCH_WARPS - 1) / MARCH_WARPS;
    march_fault_row_kernel<Real><<<blocks, 32 * MARCH_WARPS, 0, s>>>(patches, rows0, n0, rows1, n1, mc);
    return cudaGetLastError();
  }
  // resident warps of marching kernel g (0 in-plane, 1 antiplane, 2 in-plane
  // with the fused plastic return) over the device, for the scheme form fixed
  // (march_scheme_fixed) or read at run time
  static int march_slots(int g, bool fixed) {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
      return 0;
    int b;
    if (g == 0) b = fixed ? march_blocks<0, false, MARCH_SCH_PPM_PRIM>() : march_blocks<0, false, MARCH_SCH_RUNTIME>();
    else if (g == 2) b = fixed ? march_blocks<0, true, MARCH_SCH_PPM_PRIM>() : march_blocks<0, true, MARCH_SCH_RUNTIME>();
    else b = fixed ? march_blocks<1, false, MARCH_SCH_PPM_PRIM>() : march_blocks<1, false, MARCH_SCH_RUNTIME>();
    return b * sms * MARCH_WARPS;
  }
};

}  // namespace tmk

#define TMK_INSTANTIATE_LAUNCH(REAL, TXV, TYV, NTV)                                                          \
  namespace tmk {                                                                                            \
  template <> const int Launch<REAL>::TX = TXV;                                                             \
  template <> const int Launch<REAL>::TY = TYV;                                                             \
  template <> cudaError_t Launch<REAL>::fault(const PatchDev<REAL>* p, const int* fp, int nf, int mf,        \
                                              const DevParams* prm, double t, DevStatus* st, bool pdl,       \
                                              int seg, cudaStream_t s) {                                     \
    return LaunchImpl<REAL, TXV, TYV, NTV>::fault(p, fp, nf, mf, prm, t, st, pdl, seg, s);                   \
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
  template <> int Launch<REAL>::volume_box_x() { return LaunchImpl<REAL, TXV, TYV, NTV>::box_x(); }          \
  template <> int Launch<REAL>::volume_box_y() { return LaunchImpl<REAL, TXV, TYV, NTV>::box_y(); }          \
  template <> cudaError_t Launch<REAL>::plastic(const PatchDev<REAL>* p, const TileDev* tl, int nt,         \
                                                const DevParams* prm, cudaStream_t s) {                     \
    return LaunchImpl<REAL, TXV, TYV, NTV>::plastic(p, tl, nt, prm, s);                                      \
  }                                                                                                          \
  template <> cudaError_t Launch<REAL>::march(int g, const PatchDev<REAL>* p, const MarchItem* it, int n,    \
                                              const MarchConst<REAL>& mc, bool pdl, cudaStream_t s) {      \
    return LaunchImpl<REAL, TXV, TYV, NTV>::march(g, p, it, n, mc, pdl, s);                                  \
  }                                                                                                          \
  template <> cudaError_t Launch<REAL>::march_fault_rows(const PatchDev<REAL>* p, const MarchItem* r0,      \
                                                         int n0, const MarchItem* r1, int n1,              \
                                                         const MarchConst<REAL>& mc, cudaStream_t s) {     \
    return LaunchImpl<REAL, TXV, TYV, NTV>::march_fault_rows(p, r0, n0, r1, n1, mc, s);                      \
  }                                                                                                          \
  template <> int Launch<REAL>::march_slots(int g, bool fx) {                                               \
    return LaunchImpl<REAL, TXV, TYV, NTV>::march_slots(g, fx);                                              \
  }                                                                                                          \
  template <> int Launch<REAL>::march_warps() { return MARCH_WARPS; }                                        \
  template <> const void* Launch<REAL>::fault_entry(int seg) {                                               \
    return seg == FAULT_SEG_SMALL ? (const void*)fault_kernel<REAL, FAULT_SEG_SMALL, FAULT_THREADS_SMALL>     \
                                  : (const void*)fault_kernel<REAL, FAULT_SEG, FAULT_THREADS>;               \
  }                                                                                                          \
  }
