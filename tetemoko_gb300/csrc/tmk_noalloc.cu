// tmk_noalloc.cu -- tmk_patch_update_state_noalloc: the patch step of
// tmk_patch_update_state for callers that cannot allocate device memory while
// they step (a driver whose memory pool already holds the GPU's memory, or one
// that cannot accept the device-wide synchronisation of cudaMalloc/cudaFree in
// the middle of a time step).  Its temporaries -- the updated-state FAB, the
// fault-face buffers and the launch descriptors -- live in one fixed device
// array defined in this file; nothing here allocates.
#include <cuda_runtime.h>
#include <algorithm>
#include <mutex>

#include "../../include/tetemoko_gb300.h"
#include "tmk_kernels.cuh"
#include "tmk_launch.h"

namespace tmk {
struct CtxView {
  const DevParams* dp;
  DevStatus* st;
  int fault_law;
  int nb;
  double max_speed;
};
CtxView context_view(const tmk_context* c);
}  // namespace tmk

namespace {

// The scratch of every call on a device.  Its name is only a host-side handle:
// host code must use the address returned by cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_noalloc_scratch[TMK_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_addr[kMaxDevices] = {};
unsigned long long g_ctx[kMaxDevices] = {};   // the context the cached address belongs to

// Unique id of the calling thread's current CUDA context (cuCtxGetId ids are
// never reused within a process), or 0 when it cannot be had.  The driver
// calls are reached through the runtime's entry-point query, so the library
// does not link libcuda.  Call with g_mu held.
unsigned long long current_context_id() {
  typedef int (*GetCurrent)(void**);
  typedef int (*GetId)(void*, unsigned long long*);
  static bool queried = false;
  static GetCurrent get_current = nullptr;
  static GetId get_id = nullptr;
  if (!queried) {
    queried = true;
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = (GetCurrent)f;
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = (GetId)f;
  }
  void* ctx = nullptr;
  unsigned long long id = 0;
  if (get_current && get_id && get_current(&ctx) == 0 && ctx && get_id(ctx, &id) == 0) return id;
  return 0;
}

// Device address of the scratch in the current device's context.  The first
// call in a context looks it up (with that device current) and caches it; a
// new context on the device (after cudaDeviceReset, the module and its array
// are loaded again, possibly elsewhere) looks it up again.
tmk_status scratch_address(void** out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess) return TMK_ERR_CUDA;
  if (dev < 0 || dev >= kMaxDevices) return TMK_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> lk(g_mu);
  const unsigned long long id = current_context_id();
  if (!g_addr[dev] || id == 0 || id != g_ctx[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || p == nullptr) return TMK_ERR_CUDA;
    g_addr[dev] = p;
    g_ctx[dev] = current_context_id();   // the lookup made the device's primary context current
  }
  *out = g_addr[dev];
  return TMK_OK;
}

size_t up256(size_t n) { return (n + 255) & ~(size_t)255; }

// Writes the patch descriptor, the fault-patch index and the tile list of the
// valid box into the scratch (replacing the host-to-device copies of the
// allocating entry point).
__global__ void noalloc_setup_kernel(tmk::PatchDev<double> pd, tmk::PatchDev<double>* dpd, int* fault_idx,
                                     tmk::TileDev* tiles, int TX, int TY) {
  const int nx = pd.vhi0 - pd.vlo0 + 1, ny = pd.vhi1 - pd.vlo1 + 1;
  const int ntx = (nx + TX - 1) / TX, nty = (ny + TY - 1) / TY;
  if (blockIdx.x == 0 && threadIdx.x == 0) { *dpd = pd; *fault_idx = 0; }
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < ntx * nty; t += gridDim.x * blockDim.x) {
    tmk::TileDev tl;
    tl.patch = 0;
    tl.x0 = pd.vlo0 + (t % ntx) * TX;
    tl.y0 = pd.vlo1 + (t / ntx) * TY;
    tl.nx = min(TX, pd.vhi0 - tl.x0 + 1);
    tl.ny = min(TY, pd.vhi1 - tl.y0 + 1);
    tiles[t] = tl;
  }
}

}  // namespace

#define TMK_CU(call)                            \
  do {                                          \
    if ((call) != cudaSuccess) return TMK_ERR_CUDA; \
  } while (0)

extern "C" tmk_status tmk_patch_update_state_noalloc(tmk_context* c, const tmk_fab* U, const tmk_fab* B,
                                                     const tmk_fab* Fx, const tmk_fab* Fy, const tmk_box* valid,
                                                     const tmk_box* domain, double dx, double time, double dt,
                                                     double* max_wave_speed, void* stream) {
  if (!c || !U || !valid || !domain || !U->data) return TMK_ERR_BAD_DESC;
  const tmk_box& v = *valid;
  const tmk_box& d = *domain;
  if (v.lo[0] > v.hi[0] || v.lo[1] > v.hi[1] || d.lo[0] > d.hi[0] || d.lo[1] > d.hi[1]) return TMK_ERR_BAD_DESC;
  if (v.lo[0] < d.lo[0] || v.lo[1] < d.lo[1] || v.hi[0] > d.hi[0] || v.hi[1] > d.hi[1]) return TMK_ERR_BAD_DESC;
  if (U->ncomp != TMK_NCOMP || !(dx > 0) || !(dt > 0)) return TMK_ERR_BAD_DESC;
  // U must cover the valid box grown by 3 cells, within the domain
  for (int k = 0; k < 2; ++k)
    if (U->lo[k] > std::max(v.lo[k] - 3, d.lo[k]) || U->hi[k] < std::min(v.hi[k] + 3, d.hi[k])) return TMK_ERR_BAD_DESC;
  const tmk::CtxView cv = tmk::context_view(c);
  const bool fault = cv.fault_law != TMK_FAULT_NONE && v.lo[1] == d.lo[1];
  if (fault) {
    if (!B || !B->data || B->ncomp != cv.nb) return TMK_ERR_BAD_DESC;
    if (B->lo[0] > std::max(v.lo[0] - 1, d.lo[0]) || B->hi[0] < std::min(v.hi[0] + 1, d.hi[0])) return TMK_ERR_BAD_DESC;
  }
  const int nvx = v.hi[0] - v.lo[0] + 1, nvy = v.hi[1] - v.lo[1] + 1;
  if (Fx && (!Fx->data || Fx->ncomp != TMK_NCOMP || Fx->lo[0] != v.lo[0] || Fx->hi[0] != v.hi[0] + 1 ||
             Fx->lo[1] != v.lo[1] || Fx->hi[1] != v.hi[1]))
    return TMK_ERR_BAD_DESC;
  if (Fy && (!Fy->data || Fy->ncomp != TMK_NCOMP || Fy->lo[0] != v.lo[0] || Fy->hi[0] != v.hi[0] ||
             Fy->lo[1] != v.lo[1] || Fy->hi[1] != v.hi[1] + 1))
    return TMK_ERR_BAD_DESC;

  // layout of the scratch: descriptor | fault index | tiles | updated state | fault buffers
  const int TX = tmk::Launch<double>::TX, TY = tmk::Launch<double>::TY;
  const int ntiles = ((nvx + TX - 1) / TX) * ((nvy + TY - 1) / TY);
  const int anx = U->hi[0] - U->lo[0] + 1, any = U->hi[1] - U->lo[1] + 1;
  const size_t ucount = (size_t)TMK_NCOMP * anx * any;
  const size_t off_pd = 0;
  const size_t off_fi = up256(off_pd + sizeof(tmk::PatchDev<double>));
  const size_t off_tl = up256(off_fi + sizeof(int));
  const size_t off_u = up256(off_tl + (size_t)ntiles * sizeof(tmk::TileDev));
  const size_t off_first = up256(off_u + ucount * sizeof(double));
  const size_t off_ff = up256(off_first + (size_t)TMK_NCOMP * (nvx + 2) * sizeof(double));
  const size_t total = up256(off_ff + (size_t)TMK_NCOMP * nvx * sizeof(double));
  if (total > (size_t)TMK_NOALLOC_SCRATCH_BYTES) return TMK_ERR_TOO_LARGE;

  void* sp = nullptr;
  tmk_status st = scratch_address(&sp);
  if (st != TMK_OK) return st;
  char* base = (char*)sp;
  cudaStream_t s = (cudaStream_t)stream;

  tmk::PatchDev<double> pd;
  memset(&pd, 0, sizeof(pd));
  pd.Uin = U->data;
  pd.Uout = (double*)(base + off_u);
  pd.alo0 = U->lo[0]; pd.alo1 = U->lo[1]; pd.anx = anx; pd.any = any;
  pd.vlo0 = v.lo[0]; pd.vlo1 = v.lo[1]; pd.vhi0 = v.hi[0]; pd.vhi1 = v.hi[1];
  pd.dlo0 = d.lo[0]; pd.dlo1 = d.lo[1]; pd.dhi0 = d.hi[0]; pd.dhi1 = d.hi[1];
  pd.dx = dx; pd.dt = dt; pd.scen = 0;
  pd.plastic = 0;
  pd.fault = fault ? 1 : 0;
  if (fault) { pd.B = B->data; pd.blo0 = B->lo[0]; pd.bnx = B->hi[0] - B->lo[0] + 1; }
  pd.first = (double*)(base + off_first);
  pd.ffault = (double*)(base + off_ff);
  pd.nfirst = nvx + 2;
  pd.Fx = Fx ? Fx->data : nullptr;
  pd.Fy = Fy ? Fy->data : nullptr;

  tmk::PatchDev<double>* dpd = (tmk::PatchDev<double>*)(base + off_pd);
  int* dfi = (int*)(base + off_fi);
  tmk::TileDev* dtl = (tmk::TileDev*)(base + off_tl);
  const int sblocks = std::min(1024, std::max(1, (ntiles + 255) / 256));
  noalloc_setup_kernel<<<sblocks, 256, 0, s>>>(pd, dpd, dfi, dtl, TX, TY);
  TMK_CU(cudaGetLastError());
  if (Fx) TMK_CU(cudaMemsetAsync(Fx->data, 0, (size_t)TMK_NCOMP * (nvx + 1) * nvy * sizeof(double), s));
  if (Fy) TMK_CU(cudaMemsetAsync(Fy->data, 0, (size_t)TMK_NCOMP * nvx * (nvy + 1) * sizeof(double), s));
  if (fault) TMK_CU(tmk::Launch<double>::fault(dpd, dfi, 1, nvx, cv.dp, time, cv.st, false, tmk::FAULT_SEG, s));
  TMK_CU(tmk::Launch<double>::volume(dpd, dtl, ntiles, cv.dp, s));
  for (int sd = 0; sd < 2; ++sd)
    TMK_CU(tmk::copy_valid(pd.Uout, U->data, pd.alo0, pd.alo1, anx, any, pd.vlo0, pd.vlo1, pd.vhi0, pd.vhi1,
                           11 * sd, tmk::NSIDE, s));
  if (max_wave_speed) *max_wave_speed = cv.max_speed;
  return TMK_OK;
}
