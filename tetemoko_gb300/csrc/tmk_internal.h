// tmk_internal.h -- host-side objects shared by the translation units that
// implement the C ABI (tmk_capi.cu: contexts, patches, levels; tmk_amr.cu:
// coarse-fine coupling and the AMR hierarchy).
#pragma once
#include <cuda_runtime.h>
#include <algorithm>
#include <vector>

#include "../../include/tetemoko_gb300.h"
#include "tmk_kernels.cuh"
#include "tmk_march.cuh"
#include "tmk_launch.h"

#define TMK_CU(call)                                   \
  do {                                                 \
    cudaError_t e_ = (call);                           \
    if (e_ != cudaSuccess) return TMK_ERR_CUDA;        \
  } while (0)

namespace tmk_host {

inline bool box_ok(const tmk_box& b) { return b.lo[0] <= b.hi[0] && b.lo[1] <= b.hi[1]; }
inline bool box_contains(const tmk_box& a, const tmk_box& b) {
  return a.lo[0] <= b.lo[0] && a.lo[1] <= b.lo[1] && a.hi[0] >= b.hi[0] && a.hi[1] >= b.hi[1];
}
inline bool box_has(const tmk_box& a, int i, int j) {
  return i >= a.lo[0] && i <= a.hi[0] && j >= a.lo[1] && j <= a.hi[1];
}
inline tmk_box box_grow(tmk_box b, int n) { b.lo[0] -= n; b.lo[1] -= n; b.hi[0] += n; b.hi[1] += n; return b; }
inline tmk_box box_isect(tmk_box a, const tmk_box& b) {
  for (int d = 0; d < 2; ++d) { a.lo[d] = std::max(a.lo[d], b.lo[d]); a.hi[d] = std::min(a.hi[d], b.hi[d]); }
  return a;
}

template <typename T>
cudaError_t dalloc(T** p, size_t n) { return cudaMalloc((void**)p, n * sizeof(T) + 16); }

inline size_t real_size(int prec) { return prec == TMK_PREC_MIXED ? sizeof(float) : sizeof(double); }

struct LevelPatch {
  tmk_box valid, alloc;
  tmk_box domain;           // the patch's problem domain (ensembles: its scenario's)
  int scen = 0;             // scenario of the patch (index into the level's parameters)
  int fault = 0;
  void* U[2] = {nullptr, nullptr};
  double* B = nullptr;
  double* Bold = nullptr;   // fault data at the start of the step (levels with a finer level)
  int blo = 0, bnx = 0;
  double* first = nullptr;
  double* ffault = nullptr;
  double* fric = nullptr;   // per-face rate-and-state a, b, L (3 planes of bnx), if set
};

struct CFLink;   // coarse-fine coupling of a level with its coarser level (tmk_amr.cu)

// A TMA tensor map (128 bytes) of a FAB seen as a 3-D tensor (x, y,
// component) with element size `elem`, for the tile kernel's staged box of
// box_x x box_y cells of one side's 11 components.  False (map untouched) when
// the driver's encoder is not available or the FAB's base or row pitch is not
// 16-byte aligned: the kernel then loads element by element.
bool encode_fab_map(void* map, const void* data, int elem, int anx, int any, int box_x, int box_y);

}  // namespace tmk_host

struct tmk_context_s {
  tmk::DevParams hp;
  tmk::DevParams* dp = nullptr;
  tmk_scheme scheme;
  int nb = 0;
  // patch-level scratch (grown on demand)
  void* scratch = nullptr;
  size_t scratch_bytes = 0;
  tmk::DevStatus* dstatus = nullptr;
  // second stream and events of the 3-D step's overlapped schedule (made by
  // the first 3-D step of a patch with fault faces)
  cudaStream_t side = nullptr;
  cudaEvent_t side_ev[6] = {};
};

struct tmk_level_s {
  tmk_context* ctx = nullptr;              // the (first) scenario's context
  int nscen = 1;                           // scenarios of an ensemble level
  tmk_tuning tune;                         // work-list shapes and kernel variants
  int graphs = 0;                          // recorded graphs that launch this level's kernels
  tmk_stations* stations = nullptr;        // recorded after each step (postTimeStep's writeStationLevel)
  tmk::DevParams* dparams = nullptr;       // device parameters per scenario (ctx->dp for one)
  tmk_box domain;
  double dx = 0;
  int prec = TMK_PREC_FP64;
  std::vector<tmk_host::LevelPatch> patches;
  void* dpatch[2] = {nullptr, nullptr};   // PatchDev arrays, parity 0 (U0->U1) and 1 (U1->U0)
  unsigned char* dtmaps = nullptr;         // TMA tensor maps of each patch's buffers: [parity][patch], 128 B each
  std::vector<char> tmap_ok;               // per patch: its buffers have tensor maps
  std::vector<char> hpatch[2];
  std::vector<tmk::TileDev> htiles;        // tile list (host copy; capture ranges rewritten by the AMR links)
  tmk::TileDev* dtiles = nullptr;
  int ntiles = 0;
  int march = 0;                           // column-marching volume kernel
  int march_allowed = 0;                   // the scheme selects it (captures force the tile kernel)
  tmk::MarchItem* ditems[2] = {nullptr, nullptr};   // work lists of the in-plane / antiplane kernels
  int nitems[2] = {0, 0};
  tmk::MarchItem* dfrows[2] = {nullptr, nullptr};   // their fault-row items (row 0 finished after the fault kernel)
  int nfrows[2] = {0, 0};
  std::vector<tmk::MarchItem> hitems[2], hfrows[2];  // host copies (capture ranges rewritten by the AMR links)
  int4* dmcap[2] = {nullptr, nullptr};              // coarse-fine faces the marching items store
  void* stash[2] = {nullptr, nullptr};              // row-0 intermediates of those items
  int* dfault = nullptr;
  int nfault = 0, max_faces = 0;
  tmk::CopyDev* dcopies = nullptr;
  int ncopies = 0;
  tmk::CopyDev* dbcopies = nullptr;
  int nbcopies = 0;
  double** dbptr = nullptr;
  int* dblo = nullptr;
  int* dbnx = nullptr;
  double* stage = nullptr;                 // FP64 staging for set/get of the mixed form
  size_t stage_count = 0;
  // put/take of a pinned host FAB in the mixed form: the copy-engine stream
  // and one event per group of components (created on first use)
  cudaStream_t xfer = nullptr;
  cudaEvent_t xfer_ev[6] = {};
  int parity = 0;
  double cur_dt = -1.0;
  std::vector<void*> allocs;
  // with the fused plastic return the fault kernel runs on a side stream
  // forked from the step's stream and joined before the fault rows are finished
  cudaStream_t side = nullptr;
  cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
  // per-launch timing (tmk_level_profile)
  std::vector<cudaEvent_t> ev;            // 4 events per recorded step
  int prof_on = 0, prof_max = 0, prof_n = 0;
  // coarse-fine coupling
  tmk_host::CFLink* coarser = nullptr;    // owned: coupling with the next coarser level
  tmk_host::CFLink* finer = nullptr;      // the next finer level's coupling (owned by that level)
  double* cap = nullptr;                  // captured face fluxes, 22 doubles per slot
  int ncap = 0;
  int4* dcaplist = nullptr;               // (dir, i, j, slot) per captured face, grouped by tile
  std::vector<void*> cap_allocs;
};

namespace tmk_host {
// The level's state (each patch's input buffer and fault data) and its
// context's status word, saved on the device for the autotuner's trials.
struct LevelSnapshot {
  LevelSnapshot() = default;
  LevelSnapshot(const LevelSnapshot&) = delete;
  LevelSnapshot& operator=(const LevelSnapshot&) = delete;
  void* buf = nullptr;
  std::vector<size_t> uoff, ubytes, boff, bbytes;
  size_t soff = 0;
  int parity = 0;
  tmk_status save(tmk_level_s* L) {
    size_t n = 0;
    const size_t rs = real_size(L->prec);
    for (const LevelPatch& lp : L->patches) {
      const size_t ub = (size_t)TMK_NCOMP * (lp.alloc.hi[0] - lp.alloc.lo[0] + 1) * (lp.alloc.hi[1] - lp.alloc.lo[1] + 1) * rs;
      const size_t bb = lp.B ? (size_t)L->ctx->nb * lp.bnx * sizeof(double) : 0;
      uoff.push_back(n); ubytes.push_back(ub); n += (ub + 255) / 256 * 256;
      boff.push_back(n); bbytes.push_back(bb); n += (bb + 255) / 256 * 256;
    }
    soff = n;
    n += sizeof(tmk::DevStatus);
    TMK_CU(cudaMalloc(&buf, n));
    parity = L->parity;
    char* b = (char*)buf;
    for (size_t p = 0; p < L->patches.size(); ++p) {
      const LevelPatch& lp = L->patches[p];
      TMK_CU(cudaMemcpy(b + uoff[p], lp.U[parity], ubytes[p], cudaMemcpyDeviceToDevice));
      if (bbytes[p]) TMK_CU(cudaMemcpy(b + boff[p], lp.B, bbytes[p], cudaMemcpyDeviceToDevice));
    }
    TMK_CU(cudaMemcpy(b + soff, L->ctx->dstatus, sizeof(tmk::DevStatus), cudaMemcpyDeviceToDevice));
    TMK_CU(cudaDeviceSynchronize());
    return TMK_OK;
  }
  tmk_status restore(tmk_level_s* L) {
    TMK_CU(cudaDeviceSynchronize());
    L->parity = parity;
    char* b = (char*)buf;
    for (size_t p = 0; p < L->patches.size(); ++p) {
      const LevelPatch& lp = L->patches[p];
      TMK_CU(cudaMemcpy(lp.U[parity], b + uoff[p], ubytes[p], cudaMemcpyDeviceToDevice));
      if (bbytes[p]) TMK_CU(cudaMemcpy(lp.B, b + boff[p], bbytes[p], cudaMemcpyDeviceToDevice));
    }
    TMK_CU(cudaMemcpy(L->ctx->dstatus, b + soff, sizeof(tmk::DevStatus), cudaMemcpyDeviceToDevice));
    TMK_CU(cudaDeviceSynchronize());
    return TMK_OK;
  }
  ~LevelSnapshot() { if (buf) cudaFree(buf); }
};

// tmk_regrid.cu: the station kernel of a precision (its fourth parameter is the record's time)
const void* station_entry(int prec);
// tmk_capi.cu: candidate tunings of a level for the autotuners
std::vector<tmk_tuning> tuning_candidates(const tmk_level_s* L, bool reduced);
// tmk_capi.cu
tmk_status upload_patchdev(tmk_level_s* L, cudaStream_t s);
// tmk_amr.cu: the capture lists of a level's coarse-fine faces (after its work lists change)
tmk_status rebuild_captures(tmk_level_s* L);
// tmk_amr.cu: the coarse-fine parts of a level step
tmk_status amr_pre_step(tmk_level_s* L, double time, double dt, double tco, double tcn, cudaStream_t s);
tmk_status amr_post_step(tmk_level_s* L, double dt, cudaStream_t s);
int amr_launches(const tmk_level_s* L);
void amr_release(tmk_level_s* L);
}  // namespace tmk_host
