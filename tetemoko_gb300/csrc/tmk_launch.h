// tmk_launch.h -- launch wrappers, instantiated once per volume arithmetic type
// (tmk_fp64.cu is compiled without FMA contraction for the parity form,
// tmk_fp32.cu with it for the mixed form).
#pragma once
#include <cuda_runtime.h>
#include "tmk_device.cuh"

namespace tmk {

template <typename Real> struct PatchDev;
template <typename Real> struct MarchConst;
struct TileDev;
struct CopyDev;
struct MarchItem;

template <typename Real>
struct Launch {
  static const int TX, TY;
  // one thread per fault face of every fault patch, seg faces per CTA (32 or
  // 16); pdl as for march
  static cudaError_t fault(const PatchDev<Real>* patches, const int* fault_patches, int nfault, int max_faces,
                           const DevParams* params, double time, DevStatus* st, bool pdl, int seg,
                           cudaStream_t s);
  // one CTA per (tile, side)
  static cudaError_t volume(const PatchDev<Real>* patches, const TileDev* tiles, int ntiles,
                            const DevParams* params, cudaStream_t s);
  // plastic correction of every tile's cells after the marching kernels
  static cudaError_t plastic(const PatchDev<Real>* patches, const TileDev* tiles, int ntiles,
                             const DevParams* params, cudaStream_t s);
  // same-level ghost exchange of components [c0, c0+ncomp) into the input buffers
  static cudaError_t exchange(const PatchDev<Real>* patches, const CopyDev* copies, int ncopies, int c0,
                              int ncomp, cudaStream_t s);
  static size_t volume_smem();
  // the tile kernel's staged box (columns, rows) of one component: the TMA
  // tensor maps of the FABs it reads are encoded with it
  static int volume_box_x();
  static int volume_box_y();
  // column-marching volume update of component group g (0 in-plane, 1
  // antiplane): one warp per item.  pdl: the kernel may be scheduled while
  // the kernel before it in the stream still runs (programmatic dependent
  // launch; it waits for that kernel before it exits)
  static cudaError_t march(int g, const PatchDev<Real>* patches, const MarchItem* items, int nitems,
                           const MarchConst<Real>& mc, bool pdl, cudaStream_t s);
  // row 0 of the fault-row strips of both groups, after the fault kernel
  static cudaError_t march_fault_rows(const PatchDev<Real>* patches, const MarchItem* rows0, int n0,
                                      const MarchItem* rows1, int n1, const MarchConst<Real>& mc,
                                      cudaStream_t s);
  // warps of group g's marching kernel resident at once on the current device
  // (g = 2: the in-plane kernel with the fused plastic return); fixed: the
  // kernel form with the scheme fixed at compile time (PPM, primitive limiting)
  static int march_slots(int g, bool fixed);
  // warps per CTA of the marching kernels
  static int march_warps();
  // the entry of the fault kernel variant with seg faces per CTA (to find its
  // nodes in a captured graph); its fourth parameter is the step's start time
  static const void* fault_entry(int seg);
};

// FP64 <-> Real conversion of a FAB on the device
cudaError_t convert_d2f(const double* src, float* dst, size_t n, cudaStream_t s);
cudaError_t convert_f2d(const float* src, double* dst, size_t n, cudaStream_t s);
// copy of n doubles (either side may be mapped pinned host memory)
cudaError_t copy_fab(const double* src, double* dst, size_t n, cudaStream_t s);
// The components listed in comps (ncomp of them) over the valid box of two
// FABs of one shape, converted from S to D (either side may be mapped pinned
// host memory): the cells and components a level step reads and rewrites.
struct CompList { int n; int c[22]; };
cudaError_t copy_valid_comps(const double* src, float* dst, int alo0, int alo1, int anx, int any, int vlo0, int vlo1,
                             int vhi0, int vhi1, const CompList& comps, cudaStream_t s);
cudaError_t copy_valid_comps(const float* src, double* dst, int alo0, int alo1, int anx, int any, int vlo0, int vlo1,
                             int vhi0, int vhi1, const CompList& comps, cudaStream_t s);
cudaError_t copy_valid_comps(const double* src, double* dst, int alo0, int alo1, int anx, int any, int vlo0,
                             int vlo1, int vhi0, int vhi1, const CompList& comps, cudaStream_t s);
// copy components [c0, c0+ncomp) of the valid box of a FAB into another FAB of the same shape
cudaError_t copy_valid(const double* src, double* dst, int alo0, int alo1, int anx, int any, int vlo0, int vlo1,
                       int vhi0, int vhi1, int c0, int ncomp, cudaStream_t s);
cudaError_t bexchange(double* const* bptr, const int* blo, const int* bnx, const CopyDev* copies, int ncopies,
                      int nb, cudaStream_t s);
// PLASTICCORRECTION over a box of an FP64 FAB
cudaError_t plastic_fab(double* U, int alo0, int alo1, int anx, int any, int lo0, int lo1, int hi0, int hi1,
                        const DevParams* P, double dt, cudaStream_t s);

}  // namespace tmk
