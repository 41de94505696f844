// tmk_capi.cu -- the C ABI of include/tetemoko_gb300.h.
//
// Host-side objects:
//   tmk_context  per-scenario parameters (the reference's COMMON blocks) with a
//                device copy; scratch for the patch-level entry point.
//   tmk_level    device mirrors of every patch of one level (two state buffers
//                swapped each step, fault data, fault-face buffers), the tile
//                work list of the volume kernel and the exchange lists.
#include <cuda.h>            // CUtensorMap and its enums (the encoder is reached through the runtime)
#include <cuda_runtime.h>
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

#include "tmk_internal.h"

using tmk::DevParams;
using tmk::DevStatus;
using tmk::PatchDev;
using tmk::TileDev;
using tmk::CopyDev;
using namespace tmk_host;

namespace {

int device_ok() {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) return 0;
  return 1;
}

}  // namespace

extern "C" int tmk_abi_version(void) { return TMK_ABI_VERSION; }

extern "C" tmk_status tmk_context_create(const tmk_elastic_params* e, const tmk_scheme* s, const tmk_rs_params* rs,
                                         const tmk_sw_params* sw, const tmk_plastic_params* pl,
                                         tmk_context** out) {
  if (!out) return TMK_ERR_BAD_DESC;
  *out = nullptr;
  if (!e || !s) return TMK_ERR_BAD_DESC;
  if (s->normal_pred_order < 0 || s->normal_pred_order > 2) return TMK_ERR_UNSUPPORTED;
  if (s->use_char_limiting && s->use_prim_limiting) return TMK_ERR_UNSUPPORTED;  // PPMNormalPred MayDay
  for (int k = 0; k < 4; ++k)
    if (s->boundary_type[k] < 0 || s->boundary_type[k] > 2) return TMK_ERR_BAD_DESC;  // "Invalid Boundary Type"
  if (s->fault_law == TMK_FAULT_RS && !rs) return TMK_ERR_BAD_DESC;
  if (s->fault_law == TMK_FAULT_SW && !sw) return TMK_ERR_BAD_DESC;
  if (s->plasticity && !pl) return TMK_ERR_BAD_DESC;
  if (s->fault_law < 0 || s->fault_law > 2) return TMK_ERR_BAD_DESC;
  if (!(e->cs > 0) || !(e->cp >= e->cs)) return TMK_ERR_BAD_DESC;   // char transforms assume cp >= cs
  if (sw && s->fault_law == TMK_FAULT_SW && (sw->num_patches < 0 || sw->num_patches > TMK_SW_MAX_PATCHES))
    return TMK_ERR_BAD_DESC;
  if (s->volume_kernel < TMK_VOLUME_AUTO || s->volume_kernel > TMK_VOLUME_MARCH) return TMK_ERR_BAD_DESC;
  if (!device_ok()) return TMK_ERR_NO_DEVICE;
  tmk_context* c = new (std::nothrow) tmk_context_s();
  if (!c) return TMK_ERR_ALLOC;
  DevParams& P = c->hp;
  std::memset(&P, 0, sizeof(P));
  // LINELASTSETF (srcLinElast/LinElastPhysicsF.ChF:1149-1210); rho > 0 overrides G
  P.cs = e->cs; P.cp = e->cp; P.G = e->G;
  if (e->rho > 0) P.G = e->rho * e->cs * e->cs;
  P.rho = P.G / (P.cs * P.cs);
  P.lam = (P.cp * P.cp) * P.rho - 2.0 * P.G;
  P.Zs = P.rho * P.cs;
  P.Zp = P.rho * P.cp;
  P.K = P.lam + 2.0 * P.G / 3.0;
  const double bg[11] = {0, 0, 0, e->sxx0, e->syy0, e->szz0, e->sxy0, e->sxz0, e->syz0, 0, 0};
  for (int sd = 0; sd < 2; ++sd)
    for (int k = 0; k < 11; ++k) P.bg[11 * sd + k] = bg[k];
  P.order = s->normal_pred_order; P.prim_lim = s->use_prim_limiting; P.char_lim = s->use_char_limiting;
  P.fourth = s->use_fourth_order_slopes ? 1 : 0;
  for (int k = 0; k < 6; ++k) P.bc[k] = s->boundary_type[k];
  P.fault_law = s->fault_law;
  P.plasticity = s->plasticity;
  if (rs) {
    P.rs_r0 = rs->r0; P.rs_x0 = rs->x0; P.rs_nsig = rs->nsig; P.rs_a = rs->a; P.rs_b = rs->b; P.rs_V0 = rs->V0;
    P.rs_f0 = rs->f0; P.rs_L = rs->L; P.rs_fw = rs->fw; P.rs_Vw = rs->Vw; P.rs_fexp = rs->fexp;
    P.ramp_x = rs->ramp_x; P.ramp_w = rs->ramp_w; P.ramp_a = rs->ramp_a; P.ramp_Vw = rs->ramp_Vw;
    P.rs_thr = rs->rupture_threshold; P.state_law = rs->state_law;
  }
  if (sw) {
    P.sw_fs = sw->fs; P.sw_fd = sw->fd; P.sw_dw = sw->dw; P.sw_smooth = sw->smooth; P.sw_np = sw->num_patches;
    for (int k = 0; k < TMK_SW_MAX_PATCHES; ++k) { P.sw_xc[k] = sw->xc[k]; P.sw_xw[k] = sw->xw[k]; P.sw_tau[k] = sw->tau[k]; }
    P.sw_fbc0 = sw->fric_box_center[0]; P.sw_fbw0 = sw->fric_box_width[0];
    for (int k = 0; k < TMK_SW_MAX_PATCHES; ++k) { P.sw_zc[k] = sw->zc[k]; P.sw_zw[k] = sw->zw[k]; }
    P.sw_fbc1 = sw->fric_box_center[1]; P.sw_fbw1 = sw->fric_box_width[1];
    P.sw_outside = sw->outside_friction; P.sw_thr = sw->rupture_threshold;
    P.sw_off = sw->layout == TMK_SW_LAYOUT_OFFSET11 ? 11 : 9;
  }
  if (pl) { P.p_mu = pl->mu; P.p_beta = pl->beta; P.p_eta = pl->eta; P.p_b = pl->b; P.p_h = pl->h; }
  P.inv_Zs = 1.0 / P.Zs; P.inv_Zp = 1.0 / P.Zp; P.lam_r = P.lam / (P.lam + 2.0 * P.G);
  P.two_V0 = 2.0 * P.rs_V0; P.inv_2V0 = P.rs_V0 > 0 ? 1.0 / P.two_V0 : 0.0;
  P.ln_2V0 = P.rs_V0 > 0 ? std::log(P.two_V0) : 0.0;
  P.ln_halfZs = P.Zs > 0 ? std::log(0.5 * P.Zs) : 0.0;
  c->scheme = *s;
  c->nb = s->fault_law == TMK_FAULT_RS ? TMK_RS_NBDRY : (s->fault_law == TMK_FAULT_SW ? TMK_SW_NBDRY : 0);
  if (dalloc(&c->dp, 1) != cudaSuccess || dalloc(&c->dstatus, 1) != cudaSuccess) {
    cudaFree(c->dp); cudaFree(c->dstatus); delete c; return TMK_ERR_ALLOC;
  }
  if (cudaMemcpy(c->dp, &P, sizeof(P), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemset(c->dstatus, 0, sizeof(DevStatus)) != cudaSuccess) {
    cudaFree(c->dp); cudaFree(c->dstatus); delete c; return TMK_ERR_CUDA;
  }
  *out = c;
  return TMK_OK;
}

extern "C" void tmk_context_destroy(tmk_context* c) {
  if (!c) return;
  cudaFree(c->dp);
  cudaFree(c->dstatus);
  cudaFree(c->scratch);
  for (cudaEvent_t e : c->side_ev)
    if (e) cudaEventDestroy(e);
  if (c->side) cudaStreamDestroy(c->side);
  delete c;
}

extern "C" tmk_status tmk_context_constants(const tmk_context* c, double out[5]) {
  if (!c || !out) return TMK_ERR_BAD_DESC;
  out[0] = c->hp.rho; out[1] = c->hp.lam; out[2] = c->hp.K; out[3] = c->hp.Zs; out[4] = c->hp.Zp;
  return TMK_OK;
}

extern "C" tmk_status tmk_max_wave_speed(const tmk_context* c, double* speed) {
  if (!c || !speed) return TMK_ERR_BAD_DESC;
  *speed = std::max(c->hp.cs, c->hp.cp);   // MAXWAVESPEEDF
  return TMK_OK;
}

namespace {

// tiles of TX x TY over a valid box
void make_tiles(std::vector<TileDev>& out, int patch, const tmk_box& v, int TX, int TY) {
  for (int y0 = v.lo[1]; y0 <= v.hi[1]; y0 += TY)
    for (int x0 = v.lo[0]; x0 <= v.hi[0]; x0 += TX) {
      TileDev t;
      t.patch = patch; t.x0 = x0; t.y0 = y0;
      t.nx = std::min(TX, v.hi[0] - x0 + 1);
      t.ny = std::min(TY, v.hi[1] - y0 + 1);
      out.push_back(t);
    }
}

size_t align_up(size_t n) { return (n + 255) & ~(size_t)255; }

// Work items of one component group's marching kernel: strips of MARCH_COLS
// columns by runs of rows.  Each warp marches one item; the runs are sized so
// that all items fit in one wave of resident warps (`slots`): a strip gets
// max(1, floor(slots * rows / total strip-rows)) runs (at least kMinRun rows
// each, which bounds the 2-row start-up overhead).  The first run of a strip
// on the fault row waits for the fault kernel before it starts; it counts
// `wait_rows` extra rows and is shortened by as many.
constexpr int kMinRun = 16;
void make_march_items(std::vector<tmk::MarchItem>& out, std::vector<tmk::MarchItem>& fault_rows,
                      const std::vector<tmk_box>& boxes, const std::vector<int>& fault, int slots, int wait_rows,
                      int min_run) {
  long long strip_rows = 0;
  for (size_t p = 0; p < boxes.size(); ++p) {
    const tmk_box& v = boxes[p];
    const int ns = (v.hi[0] - v.lo[0] + tmk::MARCH_COLS) / tmk::MARCH_COLS;
    strip_rows += (long long)ns * (v.hi[1] - v.lo[1] + 1 + (fault[p] ? wait_rows : 0));
  }
  if (slots <= 0) slots = 1;
  for (size_t p = 0; p < boxes.size(); ++p) {
    const tmk_box& v = boxes[p];
    const int rows = v.hi[1] - v.lo[1] + 1;
    const int w = fault[p] ? wait_rows : 0;
    int k = (int)((long long)slots * (rows + w) / std::max(1LL, strip_rows));
    k = std::max(1, std::min(k, (rows + w + min_run - 1) / min_run));
    const int run = (rows + w + k - 1) / k;
    const int first = std::min(rows, std::max(4, run - w));
    for (int x0 = v.lo[0]; x0 <= v.hi[0]; x0 += tmk::MARCH_COLS)
      for (int y0 = v.lo[1]; y0 <= v.hi[1];) {
        const int len = (y0 == v.lo[1]) ? first : run;
        tmk::MarchItem m;
        m.patch = (int)p; m.x0 = x0; m.y0 = y0; m.y1 = std::min(y0 + len - 1, v.hi[1]);
        m.fslot = -1;
        m.cap0 = 0;
        m.ncap = 0;
        if (fault[p] && y0 == v.lo[1]) {       // row 0 waits for the fault kernel: finished later
          m.fslot = (int)fault_rows.size();
          fault_rows.push_back(m);
        }
        out.push_back(m);
        y0 = m.y1 + 1;
      }
  }
}

// Row-equivalents a fault-row item waits for the fault kernel (0: no marching
// item waits, row 0 of the fault patches is finished after the fault kernel),
// and the antiplane CTAs each fault-kernel CTA keeps from being resident (the
// fault kernel runs beside the antiplane kernel; measured best at 1).
constexpr int kFaultWaitRows = 0;
constexpr int kFaultDisplace = 1;

// the marching kernels implement the PPM and CTU predictors; PLM runs the tile kernel
bool uses_march(const tmk_scheme& s) { return s.volume_kernel != TMK_VOLUME_TILE && s.normal_pred_order != 1; }

tmk_tuning default_tuning(int march_allowed) {
  tmk_tuning t;
  t.volume_kernel = march_allowed ? TMK_VOLUME_MARCH : TMK_VOLUME_TILE;
  t.march_waves[0] = t.march_waves[1] = 1;
  t.min_run = kMinRun;
  t.fault_displace = kFaultDisplace;
  t.fault_seg = tmk::FAULT_SEG;
  t.fault_first = 0;
  t.plastic_fused = 0;
  return t;
}

bool tuning_ok(const tmk_level_s* L, const tmk_tuning& t) {
  if (t.volume_kernel != TMK_VOLUME_MARCH && t.volume_kernel != TMK_VOLUME_TILE) return false;
  if (t.volume_kernel == TMK_VOLUME_MARCH && !L->march_allowed) return false;
  for (int g = 0; g < 2; ++g)
    if (t.march_waves[g] < 1 || t.march_waves[g] > 8) return false;
  if (t.min_run < 4 || t.min_run > 4096 || t.fault_displace < 0 || t.fault_displace > 4) return false;
  if (t.fault_first != 0 && t.fault_first != 1) return false;
  if (t.plastic_fused != 0 && t.plastic_fused != 1) return false;
  return t.fault_seg == tmk::FAULT_SEG || t.fault_seg == tmk::FAULT_SEG_SMALL;
}

// Free a device allocation the level owns.
template <typename T>
void level_free(tmk_level_s* L, T*& p) {
  if (!p) return;
  void* v = (void*)p;
  cudaFree(v);
  L->allocs.erase(std::remove(L->allocs.begin(), L->allocs.end(), v), L->allocs.end());
  p = nullptr;
}

// The marching work lists of both component groups under the level's tuning:
// group g's list holds about march_waves[g] waves of its kernel's resident
// warps; the antiplane kernel shares the SMs with the fault kernel, leaving
// fault_displace CTA slots per fault-kernel CTA.
tmk_status build_march_lists(tmk_level_s* L) {
  const int npatch = (int)L->patches.size();
  const tmk_tuning& tu = L->tune;
  const int seg = tu.fault_seg;
  std::vector<int> fault_flags(npatch, 0);
  std::vector<tmk_box> boxes(npatch);
  int fault_ctas = 0;
  for (int p = 0; p < npatch; ++p) {
    boxes[p] = L->patches[p].valid;
    if (L->patches[p].fault) {
      fault_flags[p] = 1;
      fault_ctas += (boxes[p].hi[0] - boxes[p].lo[0] + seg) / seg;
    }
  }
  const size_t rs = real_size(L->prec);
  const int warps = L->prec == TMK_PREC_MIXED ? tmk::Launch<float>::march_warps()
                                               : tmk::Launch<double>::march_warps();
  for (int g = 0; g < 2; ++g) {
    level_free(L, L->ditems[g]);
    level_free(L, L->dfrows[g]);
    level_free(L, L->stash[g]);
    const int gk = (g == 0 && L->ctx->scheme.plasticity && tu.plastic_fused) ? 2 : g;   // the kernel of group g
    const tmk::DevParams& hp = L->ctx->hp;
    const bool fixed = hp.order != 0 && hp.prim_lim && !hp.char_lim;   // march_scheme_fixed of the launches
    int slots = L->prec == TMK_PREC_MIXED ? tmk::Launch<float>::march_slots(gk, fixed)
                                          : tmk::Launch<double>::march_slots(gk, fixed);
    slots *= tu.march_waves[g];
    if (g == 1) slots = std::max(warps, slots - tu.fault_displace * warps * fault_ctas);
    std::vector<tmk::MarchItem> items, frows;
    make_march_items(items, frows, boxes, fault_flags, slots, g == 0 && fault_ctas ? kFaultWaitRows : 0,
                     tu.min_run);
    L->nitems[g] = (int)items.size();
    L->hitems[g] = items;
    L->hfrows[g] = frows;
    if (dalloc(&L->ditems[g], items.size()) != cudaSuccess) return TMK_ERR_ALLOC;
    L->allocs.push_back(L->ditems[g]);
    TMK_CU(cudaMemcpy(L->ditems[g], items.data(), items.size() * sizeof(tmk::MarchItem), cudaMemcpyHostToDevice));
    L->nfrows[g] = (int)frows.size();
    if (!frows.empty()) {
      if (dalloc(&L->dfrows[g], frows.size()) != cudaSuccess) return TMK_ERR_ALLOC;
      L->allocs.push_back(L->dfrows[g]);
      TMK_CU(cudaMemcpy(L->dfrows[g], frows.data(), frows.size() * sizeof(tmk::MarchItem), cudaMemcpyHostToDevice));
      const size_t bytes = frows.size() * tmk::MARCH_STASH_VECS * (g == 0 ? 6 : 3) * 32 * 2 * rs;
      if (cudaMalloc(&L->stash[g], bytes) != cudaSuccess) return TMK_ERR_ALLOC;
      L->allocs.push_back(L->stash[g]);
    }
  }
  return TMK_OK;
}

}  // namespace

bool tmk_host::encode_fab_map(void* map, const void* data, int elem, int anx, int any, int box_x, int box_y) {
  typedef CUresult (*Encode)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                             const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                             CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
  static Encode encode = nullptr;
  static bool looked = false;
  if (!looked) {
    looked = true;
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      encode = (Encode)f;
  }
  if (!encode || !data || ((uintptr_t)data % 16) != 0 || ((size_t)anx * elem) % 16 != 0) return false;
  const cuuint64_t dims[3] = {(cuuint64_t)anx, (cuuint64_t)any, (cuuint64_t)TMK_NCOMP};
  const cuuint64_t strides[2] = {(cuuint64_t)anx * elem, (cuuint64_t)anx * any * elem};
  const cuuint32_t box[3] = {(cuuint32_t)box_x, (cuuint32_t)box_y, (cuuint32_t)tmk::NSIDE};
  const cuuint32_t estr[3] = {1, 1, 1};
  CUtensorMap m;
  // cells beyond the tensor read as zero (OOB fill NONE fills zeros)
  if (encode(&m, elem == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3,
             const_cast<void*>(data), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
             CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_NONE, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) !=
      CUDA_SUCCESS)
    return false;
  std::memcpy(map, &m, sizeof(m));
  return true;
}

// ---------------------------------------------------------------- patch API
extern "C" tmk_status tmk_patch_update_state(tmk_context* c, const tmk_fab* U, const tmk_fab* B, const tmk_fab* Fx,
                                             const tmk_fab* Fy, const tmk_box* valid, const tmk_box* domain,
                                             double dx, double time, double dt, double* max_wave_speed,
                                             void* stream) {
  if (!c || !U || !valid || !domain || !U->data) return TMK_ERR_BAD_DESC;
  if (!box_ok(*valid) || !box_ok(*domain) || !box_contains(*domain, *valid)) return TMK_ERR_BAD_DESC;
  if (U->ncomp != TMK_NCOMP || !(dx > 0) || !(dt > 0)) return TMK_ERR_BAD_DESC;
  tmk_box ub; ub.lo[0] = U->lo[0]; ub.lo[1] = U->lo[1]; ub.hi[0] = U->hi[0]; ub.hi[1] = U->hi[1];
  if (!box_contains(ub, box_isect(box_grow(*valid, 3), *domain))) return TMK_ERR_BAD_DESC;
  const bool fault = c->scheme.fault_law != TMK_FAULT_NONE && valid->lo[1] == domain->lo[1];
  if (fault) {
    if (!B || !B->data || B->ncomp != c->nb) return TMK_ERR_BAD_DESC;
    int need_lo = std::max(valid->lo[0] - 1, domain->lo[0]), need_hi = std::min(valid->hi[0] + 1, domain->hi[0]);
    if (B->lo[0] > need_lo || B->hi[0] < need_hi) return TMK_ERR_BAD_DESC;
  }
  const int nvx = valid->hi[0] - valid->lo[0] + 1, nvy = valid->hi[1] - valid->lo[1] + 1;
  if (Fx && (!Fx->data || Fx->ncomp != TMK_NCOMP || Fx->lo[0] != valid->lo[0] || Fx->hi[0] != valid->hi[0] + 1 ||
             Fx->lo[1] != valid->lo[1] || Fx->hi[1] != valid->hi[1]))
    return TMK_ERR_BAD_DESC;
  if (Fy && (!Fy->data || Fy->ncomp != TMK_NCOMP || Fy->lo[0] != valid->lo[0] || Fy->hi[0] != valid->hi[0] ||
             Fy->lo[1] != valid->lo[1] || Fy->hi[1] != valid->hi[1] + 1))
    return TMK_ERR_BAD_DESC;
  cudaStream_t s = (cudaStream_t)stream;
  const int anx = U->hi[0] - U->lo[0] + 1, any = U->hi[1] - U->lo[1] + 1;
  const size_t ucount = (size_t)TMK_NCOMP * anx * any;
  std::vector<TileDev> tiles;
  make_tiles(tiles, 0, *valid, tmk::Launch<double>::TX, tmk::Launch<double>::TY);
  const int nfirst = nvx + 2;
  // scratch: Uout | first | ffault | PatchDev | tiles | fault patch index
  size_t off_u = 0;
  size_t off_first = align_up(off_u + ucount * sizeof(double));
  size_t off_ff = align_up(off_first + (size_t)TMK_NCOMP * nfirst * sizeof(double));
  size_t off_pd = align_up(off_ff + (size_t)TMK_NCOMP * nvx * sizeof(double));
  size_t off_tl = align_up(off_pd + sizeof(PatchDev<double>));
  size_t off_fp = align_up(off_tl + tiles.size() * sizeof(TileDev));
  size_t off_tm = align_up(off_fp + sizeof(int));
  size_t total = align_up(off_tm + sizeof(CUtensorMap));
  if (total > c->scratch_bytes) {
    TMK_CU(cudaStreamSynchronize(s));
    cudaFree(c->scratch);
    c->scratch = nullptr; c->scratch_bytes = 0;
    if (cudaMalloc(&c->scratch, total) != cudaSuccess) return TMK_ERR_ALLOC;
    c->scratch_bytes = total;
  }
  char* base = (char*)c->scratch;
  PatchDev<double> pd;
  std::memset(&pd, 0, sizeof(pd));
  pd.Uin = U->data;
  pd.Uout = (double*)(base + off_u);
  pd.alo0 = U->lo[0]; pd.alo1 = U->lo[1]; pd.anx = anx; pd.any = any;
  pd.vlo0 = valid->lo[0]; pd.vlo1 = valid->lo[1]; pd.vhi0 = valid->hi[0]; pd.vhi1 = valid->hi[1];
  pd.dlo0 = domain->lo[0]; pd.dlo1 = domain->lo[1]; pd.dhi0 = domain->hi[0]; pd.dhi1 = domain->hi[1];
  pd.dx = dx; pd.dt = dt; pd.scen = 0;
  pd.plastic = 0;   // LinElastLevelGodunov::plasticUpdate is a separate call (tmk_plastic_update)
  pd.fault = fault ? 1 : 0;
  if (fault) { pd.B = B->data; pd.blo0 = B->lo[0]; pd.bnx = B->hi[0] - B->lo[0] + 1; }
  pd.first = (double*)(base + off_first);
  pd.ffault = (double*)(base + off_ff);
  pd.nfirst = nfirst;
  pd.Fx = Fx ? Fx->data : nullptr;
  pd.Fy = Fy ? Fy->data : nullptr;
  pd.status = c->dstatus;
  // the tile kernel stages its tiles with TMA when U's layout allows a tensor map
  alignas(64) unsigned char tmap[sizeof(CUtensorMap)];
  const bool use_tma = encode_fab_map(tmap, U->data, (int)sizeof(double), anx, any,
                                      tmk::Launch<double>::volume_box_x(), tmk::Launch<double>::volume_box_y());
  pd.tmap = use_tma ? (const void*)(base + off_tm) : nullptr;
  const int zero = 0;
  // descriptors are staged through pageable memory: synchronous with respect to the host
  TMK_CU(cudaMemcpyAsync(base + off_pd, &pd, sizeof(pd), cudaMemcpyHostToDevice, s));
  TMK_CU(cudaMemcpyAsync(base + off_tl, tiles.data(), tiles.size() * sizeof(TileDev), cudaMemcpyHostToDevice, s));
  TMK_CU(cudaMemcpyAsync(base + off_fp, &zero, sizeof(int), cudaMemcpyHostToDevice, s));
  if (use_tma) TMK_CU(cudaMemcpyAsync(base + off_tm, tmap, sizeof(tmap), cudaMemcpyHostToDevice, s));
  if (Fx) TMK_CU(cudaMemsetAsync(Fx->data, 0, (size_t)TMK_NCOMP * (nvx + 1) * nvy * sizeof(double), s));
  if (Fy) TMK_CU(cudaMemsetAsync(Fy->data, 0, (size_t)TMK_NCOMP * nvx * (nvy + 1) * sizeof(double), s));
  const PatchDev<double>* dpd = (const PatchDev<double>*)(base + off_pd);
  if (fault)
    TMK_CU(tmk::Launch<double>::fault(dpd, (const int*)(base + off_fp), 1, nvx, c->dp, time, c->dstatus, false, tmk::FAULT_SEG, s));
  TMK_CU(tmk::Launch<double>::volume(dpd, (const TileDev*)(base + off_tl), (int)tiles.size(), c->dp, s));
  // the volume kernel writes the nine evolving components of each side;
  // lambda and gamma are left untouched, as updateState leaves them
  for (int sd = 0; sd < 2; ++sd)
    TMK_CU(tmk::copy_valid(pd.Uout, U->data, pd.alo0, pd.alo1, anx, any, pd.vlo0, pd.vlo1, pd.vhi0, pd.vhi1,
                           11 * sd, tmk::NSIDE, s));
  if (max_wave_speed) *max_wave_speed = std::max(c->hp.cs, c->hp.cp);
  return TMK_OK;
}

extern "C" tmk_status tmk_plastic_update(tmk_context* c, const tmk_fab* U, const tmk_box* box, double dt,
                                         void* stream) {
  if (!c || !U || !U->data || !box || U->ncomp != TMK_NCOMP || !box_ok(*box)) return TMK_ERR_BAD_DESC;
  tmk_box ub; ub.lo[0] = U->lo[0]; ub.lo[1] = U->lo[1]; ub.hi[0] = U->hi[0]; ub.hi[1] = U->hi[1];
  if (!box_contains(ub, *box)) return TMK_ERR_BAD_DESC;
  const int anx = U->hi[0] - U->lo[0] + 1, any = U->hi[1] - U->lo[1] + 1;
  TMK_CU(tmk::plastic_fab(U->data, U->lo[0], U->lo[1], anx, any, box->lo[0], box->lo[1], box->hi[0], box->hi[1],
                          c->dp, dt, (cudaStream_t)stream));
  return TMK_OK;
}

// ---------------------------------------------------------------- level API
namespace {

template <typename Real>
void fill_patchdev(tmk_level_s* L, int parity) {
  L->hpatch[parity].assign(L->patches.size() * sizeof(PatchDev<Real>), 0);
  PatchDev<Real>* hp = (PatchDev<Real>*)L->hpatch[parity].data();
  for (size_t p = 0; p < L->patches.size(); ++p) {
    const LevelPatch& lp = L->patches[p];
    PatchDev<Real>& d = hp[p];
    d.Uin = (const Real*)lp.U[parity];
    d.Uout = (Real*)lp.U[1 - parity];
    d.alo0 = lp.alloc.lo[0]; d.alo1 = lp.alloc.lo[1];
    d.anx = lp.alloc.hi[0] - lp.alloc.lo[0] + 1; d.any = lp.alloc.hi[1] - lp.alloc.lo[1] + 1;
    d.vlo0 = lp.valid.lo[0]; d.vlo1 = lp.valid.lo[1]; d.vhi0 = lp.valid.hi[0]; d.vhi1 = lp.valid.hi[1];
    d.dlo0 = lp.domain.lo[0]; d.dlo1 = lp.domain.lo[1]; d.dhi0 = lp.domain.hi[0]; d.dhi1 = lp.domain.hi[1];
    d.dx = L->dx; d.dt = L->cur_dt; d.scen = lp.scen;
    d.plastic = L->ctx->scheme.plasticity ? 1 : 0;
    d.fault = lp.fault;
    d.B = lp.B; d.blo0 = lp.blo; d.bnx = lp.bnx;
    d.first = lp.first; d.ffault = lp.ffault;
    d.nfirst = lp.valid.hi[0] - lp.valid.lo[0] + 3;
    d.Fx = nullptr; d.Fy = nullptr;
    d.Bold = lp.Bold;
    d.cap = L->cap;
    d.caplist = L->dcaplist;
    d.fric = lp.fric;
    d.tmap = L->tmap_ok.size() > p && L->tmap_ok[p]
                 ? (const void*)(L->dtmaps + ((size_t)parity * L->patches.size() + p) * sizeof(CUtensorMap))
                 : nullptr;
    d.status = L->ctx->dstatus;
  }
}

}  // namespace

tmk_status tmk_host::upload_patchdev(tmk_level_s* L, cudaStream_t s) {
  for (int par = 0; par < 2; ++par) {
    if (L->prec == TMK_PREC_MIXED) fill_patchdev<float>(L, par); else fill_patchdev<double>(L, par);
    // a copy from pageable memory returns once the source has been staged
    TMK_CU(cudaMemcpyAsync(L->dpatch[par], L->hpatch[par].data(), L->hpatch[par].size(), cudaMemcpyHostToDevice, s));
  }
  return TMK_OK;
}

extern "C" tmk_status tmk_level_set_fault_friction(tmk_level* L, int patch, const double* abL, int host) {
  if (!L || !abL || patch < 0 || patch >= (int)L->patches.size()) return TMK_ERR_BAD_DESC;
  LevelPatch& lp = L->patches[patch];
  if (!lp.fault || L->ctx->scheme.fault_law != TMK_FAULT_RS) return TMK_ERR_BAD_DESC;
  const size_t n = 3 * (size_t)lp.bnx;
  std::vector<double> h(n);   // staged on the host: every face's a, b, L must be positive
  TMK_CU(cudaMemcpy(h.data(), abL, n * sizeof(double), host ? cudaMemcpyHostToHost : cudaMemcpyDeviceToHost));
  for (int i = 0; i < lp.bnx; ++i)
    if (!(h[i] > 0) || !(h[lp.bnx + i] > 0) || !(h[2 * lp.bnx + i] > 0)) return TMK_ERR_BAD_DESC;
  const bool fresh = lp.fric == nullptr;
  if (fresh) {
    if (dalloc(&lp.fric, n) != cudaSuccess) return TMK_ERR_ALLOC;
    L->allocs.push_back(lp.fric);
  }
  TMK_CU(cudaMemcpy(lp.fric, h.data(), n * sizeof(double), cudaMemcpyHostToDevice));
  if (fresh && upload_patchdev(L, 0) != TMK_OK) return TMK_ERR_CUDA;
  TMK_CU(cudaDeviceSynchronize());
  return TMK_OK;
}

extern "C" tmk_status tmk_level_get_fault_friction(const tmk_level* L, int patch, double* abL, int host,
                                                   int* present) {
  if (!L || !abL || !present || patch < 0 || patch >= (int)L->patches.size()) return TMK_ERR_BAD_DESC;
  const LevelPatch& lp = L->patches[patch];
  *present = lp.fric ? 1 : 0;
  if (!lp.fric) return TMK_OK;
  TMK_CU(cudaMemcpy(abL, lp.fric, 3 * (size_t)lp.bnx * sizeof(double),
                    host ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice));
  return TMK_OK;
}

extern "C" void tmk_level_destroy(tmk_level* L) {
  if (!L) return;
  cudaDeviceSynchronize();
  amr_release(L);
  for (void* p : L->allocs) cudaFree(p);
  for (void* p : L->cap_allocs) cudaFree(p);
  for (cudaEvent_t e : L->ev) cudaEventDestroy(e);
  if (L->fork_ev) cudaEventDestroy(L->fork_ev);
  if (L->join_ev) cudaEventDestroy(L->join_ev);
  if (L->side) cudaStreamDestroy(L->side);
  for (cudaEvent_t e : L->xfer_ev)
    if (e) cudaEventDestroy(e);
  if (L->xfer) cudaStreamDestroy(L->xfer);
  delete L;
}

namespace {

// A level whose patch p covers boxes[p] of domain pdom[p] and belongs to
// scenario pscen[p] (context ctxs[pscen[p]]): one scenario for a level of the
// reference, several for an ensemble.
tmk_status level_create_impl(tmk_context* const* ctxs, int nscen, const tmk_box* pdom, const int* pscen,
                             double dx, int npatch, const tmk_box* boxes, tmk_level** out) {
  tmk_context* c = ctxs[0];
  // patches must be valid, inside their domain and disjoint within a scenario
  for (int p = 0; p < npatch; ++p) {
    if (pscen[p] < 0 || pscen[p] >= nscen) return TMK_ERR_BAD_DESC;
    if (!box_ok(pdom[p]) || pdom[p].hi[1] - pdom[p].lo[1] < 2) return TMK_ERR_BAD_DESC;  // fault stencil: 3 rows
    if (!box_ok(boxes[p]) || !box_contains(pdom[p], boxes[p])) return TMK_ERR_BAD_DESC;
    for (int q = 0; q < p; ++q) {
      tmk_box x = box_isect(boxes[p], boxes[q]);
      if (pscen[q] == pscen[p] && box_ok(x)) return TMK_ERR_BAD_DESC;
    }
  }
  tmk_level_s* L = new (std::nothrow) tmk_level_s();
  if (!L) return TMK_ERR_ALLOC;
  L->ctx = c; L->domain = pdom[0]; L->dx = dx; L->prec = c->scheme.precision;
  L->nscen = nscen;
  L->dparams = c->dp;
  L->patches.resize(npatch);
  const size_t rs = real_size(L->prec);
  const int nb = c->nb;
  std::vector<TileDev> tiles;
  std::vector<int> fault_idx;
  const int TX = L->prec == TMK_PREC_MIXED ? tmk::Launch<float>::TX : tmk::Launch<double>::TX;
  const int TY = L->prec == TMK_PREC_MIXED ? tmk::Launch<float>::TY : tmk::Launch<double>::TY;
  auto fail = [&](tmk_status st) { tmk_level_destroy(L); return st; };
  size_t max_count = 0;
  if (nscen > 1) {
    if (dalloc(&L->dparams, (size_t)nscen) != cudaSuccess) return fail(TMK_ERR_ALLOC);
    L->allocs.push_back(L->dparams);
    for (int k = 0; k < nscen; ++k)
      TMK_CU(cudaMemcpy(L->dparams + k, &ctxs[k]->hp, sizeof(DevParams), cudaMemcpyHostToDevice));
  }
  for (int p = 0; p < npatch; ++p) {
    LevelPatch& lp = L->patches[p];
    lp.valid = boxes[p];
    lp.domain = pdom[p];
    lp.scen = pscen[p];
    lp.alloc = box_grow(boxes[p], TMK_NGHOST);
    const int anx = lp.alloc.hi[0] - lp.alloc.lo[0] + 1, any = lp.alloc.hi[1] - lp.alloc.lo[1] + 1;
    const size_t count = (size_t)TMK_NCOMP * anx * any;
    max_count = std::max(max_count, count);
    for (int k = 0; k < 2; ++k) {
      if (cudaMalloc(&lp.U[k], count * rs) != cudaSuccess) return fail(TMK_ERR_ALLOC);
      L->allocs.push_back(lp.U[k]);
      if (cudaMemset(lp.U[k], 0, count * rs) != cudaSuccess) return fail(TMK_ERR_CUDA);
    }
    lp.fault = (c->scheme.fault_law != TMK_FAULT_NONE && boxes[p].lo[1] == pdom[p].lo[1]) ? 1 : 0;
    if (lp.fault) {
      lp.blo = boxes[p].lo[0] - TMK_NGHOST;
      lp.bnx = boxes[p].hi[0] - boxes[p].lo[0] + 1 + 2 * TMK_NGHOST;
      const int nv = boxes[p].hi[0] - boxes[p].lo[0] + 1;
      if (dalloc(&lp.B, (size_t)nb * lp.bnx) != cudaSuccess) return fail(TMK_ERR_ALLOC);
      L->allocs.push_back(lp.B);
      if (dalloc(&lp.first, (size_t)TMK_NCOMP * (nv + 2)) != cudaSuccess) return fail(TMK_ERR_ALLOC);
      L->allocs.push_back(lp.first);
      if (dalloc(&lp.ffault, (size_t)TMK_NCOMP * nv) != cudaSuccess) return fail(TMK_ERR_ALLOC);
      L->allocs.push_back(lp.ffault);
      cudaMemset(lp.B, 0, (size_t)nb * lp.bnx * sizeof(double));
      cudaMemset(lp.ffault, 0, (size_t)TMK_NCOMP * nv * sizeof(double));
      fault_idx.push_back(p);
      L->max_faces = std::max(L->max_faces, nv);
    }
    make_tiles(tiles, p, boxes[p], TX, TY);
  }
  // fault-row tiles first so that their CTAs start early
  std::stable_sort(tiles.begin(), tiles.end(), [&](const TileDev& a, const TileDev& b) {
    return (a.y0 == pdom[a.patch].lo[1]) > (b.y0 == pdom[b.patch].lo[1]);
  });
  // same-level exchange lists: ghost cells of p covered by valid cells of q
  std::vector<CopyDev> copies, bcopies;
  for (int p = 0; p < npatch; ++p)
    for (int q = 0; q < npatch; ++q) {
      if (p == q || pscen[p] != pscen[q]) continue;
      tmk_box g = box_isect(box_isect(L->patches[p].alloc, boxes[q]), pdom[p]);
      if (box_ok(g)) {
        CopyDev cd; cd.src = q; cd.dst = p; cd.lo0 = g.lo[0]; cd.lo1 = g.lo[1]; cd.hi0 = g.hi[0]; cd.hi1 = g.hi[1];
        copies.push_back(cd);
      }
      if (L->patches[p].fault && L->patches[q].fault) {
        int lo = std::max(L->patches[p].blo, boxes[q].lo[0]);
        int hi = std::min(L->patches[p].blo + L->patches[p].bnx - 1, boxes[q].hi[0]);
        if (lo <= hi) {
          CopyDev cd; cd.src = q; cd.dst = p; cd.lo0 = lo; cd.hi0 = hi; cd.lo1 = cd.hi1 = pdom[p].lo[1];
          bcopies.push_back(cd);
        }
      }
    }
  L->ntiles = (int)tiles.size();
  L->nfault = (int)fault_idx.size();
  L->ncopies = (int)copies.size();
  L->nbcopies = (int)bcopies.size();
  size_t pds = L->prec == TMK_PREC_MIXED ? sizeof(PatchDev<float>) : sizeof(PatchDev<double>);
  for (int k = 0; k < 2; ++k) {
    if (cudaMalloc(&L->dpatch[k], pds * npatch) != cudaSuccess) return fail(TMK_ERR_ALLOC);
    L->allocs.push_back(L->dpatch[k]);
  }
  // TMA tensor maps of every patch's two state buffers, for the tile kernel
  {
    const int rs_ = (int)real_size(L->prec);
    const int bx = L->prec == TMK_PREC_MIXED ? tmk::Launch<float>::volume_box_x() : tmk::Launch<double>::volume_box_x();
    const int by = L->prec == TMK_PREC_MIXED ? tmk::Launch<float>::volume_box_y() : tmk::Launch<double>::volume_box_y();
    std::vector<unsigned char> h((size_t)2 * npatch * sizeof(CUtensorMap), 0);
    L->tmap_ok.assign(npatch, 1);
    for (int k = 0; k < 2; ++k)
      for (int p = 0; p < npatch; ++p) {
        const LevelPatch& lp = L->patches[p];
        const int anx = lp.alloc.hi[0] - lp.alloc.lo[0] + 1, any = lp.alloc.hi[1] - lp.alloc.lo[1] + 1;
        if (!encode_fab_map(h.data() + ((size_t)k * npatch + p) * sizeof(CUtensorMap), lp.U[k], rs_, anx, any, bx, by))
          L->tmap_ok[p] = 0;
      }
    if (cudaMalloc(&L->dtmaps, h.size()) != cudaSuccess) return fail(TMK_ERR_ALLOC);
    L->allocs.push_back(L->dtmaps);
    TMK_CU(cudaMemcpy(L->dtmaps, h.data(), h.size(), cudaMemcpyHostToDevice));
  }
  if (dalloc(&L->dtiles, tiles.size()) != cudaSuccess) return fail(TMK_ERR_ALLOC);
  L->allocs.push_back(L->dtiles);
  L->htiles = tiles;
  L->march_allowed = uses_march(c->scheme) ? 1 : 0;
  L->march = L->march_allowed;
  L->tune = default_tuning(L->march_allowed);
  if (L->march_allowed) {
    tmk_status st = build_march_lists(L);
    if (st != TMK_OK) return fail(st);
  }
  TMK_CU(cudaMemcpy(L->dtiles, tiles.data(), tiles.size() * sizeof(TileDev), cudaMemcpyHostToDevice));
  if (L->nfault) {
    if (dalloc(&L->dfault, fault_idx.size()) != cudaSuccess) return fail(TMK_ERR_ALLOC);
    L->allocs.push_back(L->dfault);
    TMK_CU(cudaMemcpy(L->dfault, fault_idx.data(), fault_idx.size() * sizeof(int), cudaMemcpyHostToDevice));
  }
  if (L->ncopies) {
    if (dalloc(&L->dcopies, copies.size()) != cudaSuccess) return fail(TMK_ERR_ALLOC);
    L->allocs.push_back(L->dcopies);
    TMK_CU(cudaMemcpy(L->dcopies, copies.data(), copies.size() * sizeof(CopyDev), cudaMemcpyHostToDevice));
  }
  if (L->nbcopies) {
    std::vector<double*> bp(npatch, nullptr);
    std::vector<int> blo(npatch, 0), bnx(npatch, 0);
    for (int p = 0; p < npatch; ++p) { bp[p] = L->patches[p].B; blo[p] = L->patches[p].blo; bnx[p] = L->patches[p].bnx; }
    if (dalloc(&L->dbcopies, bcopies.size()) != cudaSuccess || dalloc(&L->dbptr, npatch) != cudaSuccess ||
        dalloc(&L->dblo, npatch) != cudaSuccess || dalloc(&L->dbnx, npatch) != cudaSuccess)
      return fail(TMK_ERR_ALLOC);
    L->allocs.push_back(L->dbcopies); L->allocs.push_back(L->dbptr);
    L->allocs.push_back(L->dblo); L->allocs.push_back(L->dbnx);
    TMK_CU(cudaMemcpy(L->dbcopies, bcopies.data(), bcopies.size() * sizeof(CopyDev), cudaMemcpyHostToDevice));
    TMK_CU(cudaMemcpy(L->dbptr, bp.data(), npatch * sizeof(double*), cudaMemcpyHostToDevice));
    TMK_CU(cudaMemcpy(L->dblo, blo.data(), npatch * sizeof(int), cudaMemcpyHostToDevice));
    TMK_CU(cudaMemcpy(L->dbnx, bnx.data(), npatch * sizeof(int), cudaMemcpyHostToDevice));
  }
  if (L->prec == TMK_PREC_MIXED) {
    if (dalloc(&L->stage, max_count) != cudaSuccess) return fail(TMK_ERR_ALLOC);
    L->allocs.push_back(L->stage);
    L->stage_count = max_count;
  }
  if (upload_patchdev(L, 0) != TMK_OK) return fail(TMK_ERR_CUDA);
  TMK_CU(cudaDeviceSynchronize());
  *out = L;
  return TMK_OK;
}

// the parameters an ensemble's scenarios must share: everything but friction
bool same_bulk(const tmk_context* a, const tmk_context* b) {
  const DevParams &p = a->hp, &q = b->hp;
  if (p.cs != q.cs || p.cp != q.cp || p.G != q.G || p.rho != q.rho) return false;
  for (int k = 0; k < 22; ++k) if (p.bg[k] != q.bg[k]) return false;
  const tmk_scheme &s = a->scheme, &t = b->scheme;
  if (s.normal_pred_order != t.normal_pred_order || s.use_prim_limiting != t.use_prim_limiting ||
      s.use_fourth_order_slopes != t.use_fourth_order_slopes ||
      s.use_char_limiting != t.use_char_limiting || s.fault_law != t.fault_law || s.plasticity != t.plasticity ||
      s.precision != t.precision || s.volume_kernel != t.volume_kernel)
    return false;
  for (int k = 0; k < 6; ++k) if (s.boundary_type[k] != t.boundary_type[k]) return false;
  if (s.plasticity && (p.p_mu != q.p_mu || p.p_beta != q.p_beta || p.p_eta != q.p_eta || p.p_b != q.p_b ||
                       p.p_h != q.p_h))
    return false;
  return true;
}

}  // namespace

extern "C" tmk_status tmk_level_create(tmk_context* c, const tmk_box* domain, double dx, int npatch,
                                       const tmk_box* boxes, tmk_level** out) {
  if (!out) return TMK_ERR_BAD_DESC;
  *out = nullptr;
  if (!c || !domain || !boxes || npatch <= 0 || !(dx > 0) || !box_ok(*domain)) return TMK_ERR_BAD_DESC;
  std::vector<tmk_box> pdom(npatch, *domain);
  std::vector<int> pscen(npatch, 0);
  return level_create_impl(&c, 1, pdom.data(), pscen.data(), dx, npatch, boxes, out);
}

extern "C" tmk_status tmk_ensemble_create(int nscen, tmk_context* const* ctxs, const tmk_box* domains, double dx,
                                          int npatch, const tmk_box* boxes, const int* patch_scen,
                                          tmk_level** out) {
  if (!out) return TMK_ERR_BAD_DESC;
  *out = nullptr;
  if (nscen < 1 || !ctxs || !domains || !boxes || !patch_scen || npatch <= 0 || !(dx > 0)) return TMK_ERR_BAD_DESC;
  for (int k = 0; k < nscen; ++k) {
    if (!ctxs[k] || !box_ok(domains[k])) return TMK_ERR_BAD_DESC;
    if (!same_bulk(ctxs[0], ctxs[k])) return TMK_ERR_UNSUPPORTED;
  }
  std::vector<tmk_box> pdom(npatch);
  for (int p = 0; p < npatch; ++p) {
    if (patch_scen[p] < 0 || patch_scen[p] >= nscen) return TMK_ERR_BAD_DESC;
    pdom[p] = domains[patch_scen[p]];
  }
  return level_create_impl(ctxs, nscen, pdom.data(), patch_scen, dx, npatch, boxes, out);
}

namespace {

// The device address of host memory the device can read and write directly
// (pinned memory), else null: pageable memory goes through a staging copy.
void* mapped_host(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) { cudaGetLastError(); return nullptr; }
  return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

}  // namespace

extern "C" tmk_status tmk_level_set_patch(tmk_level* L, int p, const double* U, const double* B, int host) {
  if (!L || p < 0 || p >= (int)L->patches.size() || !U) return TMK_ERR_BAD_DESC;
  LevelPatch& lp = L->patches[p];
  const size_t count = (size_t)TMK_NCOMP * (lp.alloc.hi[0] - lp.alloc.lo[0] + 1) * (lp.alloc.hi[1] - lp.alloc.lo[1] + 1);
  const cudaMemcpyKind kind = host ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
  const int k = L->parity;   // the buffer the next step reads
  // a device pointer or pinned host memory is read in place by the kernel
  const double* src = host ? (const double*)mapped_host(U) : U;
  if (L->prec == TMK_PREC_MIXED) {
    if (!src) {
      TMK_CU(cudaMemcpy(L->stage, U, count * sizeof(double), kind));
      src = L->stage;
    }
    TMK_CU(tmk::convert_d2f(src, (float*)lp.U[k], count, 0));
  } else if (src) {
    TMK_CU(tmk::copy_fab(src, (double*)lp.U[k], count, 0));
  } else {
    TMK_CU(cudaMemcpy(lp.U[k], U, count * sizeof(double), kind));
  }
  // lambda and gamma are the only planes a step without plasticity never
  // rewrites: keep them identical in the other buffer
  const size_t plane = count / TMK_NCOMP * real_size(L->prec);
  for (int c : {9, 10, 20, 21})
    TMK_CU(cudaMemcpy((char*)lp.U[1 - k] + c * plane, (char*)lp.U[k] + c * plane, plane, cudaMemcpyDeviceToDevice));
  if (lp.fault) {
    if (!B) return TMK_ERR_BAD_DESC;
    TMK_CU(cudaMemcpy(lp.B, B, (size_t)L->ctx->nb * lp.bnx * sizeof(double), kind));
  }
  TMK_CU(cudaDeviceSynchronize());
  return TMK_OK;
}

extern "C" tmk_status tmk_level_get_patch(tmk_level* L, int p, double* U, double* B, int host) {
  if (!L || p < 0 || p >= (int)L->patches.size()) return TMK_ERR_BAD_DESC;
  LevelPatch& lp = L->patches[p];
  const size_t count = (size_t)TMK_NCOMP * (lp.alloc.hi[0] - lp.alloc.lo[0] + 1) * (lp.alloc.hi[1] - lp.alloc.lo[1] + 1);
  const cudaMemcpyKind kind = host ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
  TMK_CU(cudaDeviceSynchronize());
  if (U) {
    double* dst = host ? (double*)mapped_host(U) : U;   // written in place when the device can reach it
    if (L->prec == TMK_PREC_MIXED) {
      TMK_CU(tmk::convert_f2d((const float*)lp.U[L->parity], dst ? dst : L->stage, count, 0));
      if (!dst) TMK_CU(cudaMemcpy(U, L->stage, count * sizeof(double), kind));
    } else if (dst) {
      TMK_CU(tmk::copy_fab((const double*)lp.U[L->parity], dst, count, 0));
    } else {
      TMK_CU(cudaMemcpy(U, lp.U[L->parity], count * sizeof(double), kind));
    }
  }
  if (B && lp.fault) TMK_CU(cudaMemcpy(B, lp.B, (size_t)L->ctx->nb * lp.bnx * sizeof(double), kind));
  TMK_CU(cudaDeviceSynchronize());
  return TMK_OK;
}

namespace {

// The components a step of level L reads and rewrites: the 9 evolving ones of
// each side, and lambda and gamma where the scheme has plasticity.
tmk::CompList step_comps(const tmk_level_s* L) {
  tmk::CompList cl;
  cl.n = 0;
  const bool pl = L->ctx->scheme.plasticity != 0;
  for (int c = 0; c < TMK_NCOMP; ++c)
    if (pl || (c % TMK_NSIDE_COMP) < tmk::NSIDE) cl.c[cl.n++] = c;
  return cl;
}

// Mixed form, pinned host FAB: the copy engines move the valid rows of one
// group of components between the host FAB and the FP64 staging buffer (the
// same layout) while the conversion kernel works on the group before it (put:
// copy, then convert into the state; take: convert out of the state, then
// copy).  The host link bounds both (about 210 GB/s to the device and 190 GB/s
// back on GB300, whatever the number of copy streams); the conversion kernel
// reading or writing the mapped host FAB itself reached 88-91 % of that.  The
// transfer stream starts after the work the legacy stream is ordered after.
tmk_status valid_copy_pinned(tmk_level_s* L, LevelPatch& lp, const double* in, double* out,
                             const tmk::CompList& cl) {
  constexpr int kGroups = (int)(sizeof(L->xfer_ev) / sizeof(L->xfer_ev[0]));
  if (!L->xfer) TMK_CU(cudaStreamCreateWithFlags(&L->xfer, cudaStreamNonBlocking));
  for (cudaEvent_t& e : L->xfer_ev)
    if (!e) TMK_CU(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  const int alo0 = lp.alloc.lo[0], alo1 = lp.alloc.lo[1];
  const int anx = lp.alloc.hi[0] - alo0 + 1, any = lp.alloc.hi[1] - alo1 + 1;
  const tmk_box& v = lp.valid;
  const size_t pitch = (size_t)anx * sizeof(double);
  const size_t width = (size_t)(v.hi[0] - v.lo[0] + 1) * sizeof(double);
  const size_t rows = (size_t)(v.hi[1] - v.lo[1] + 1);
  const size_t o0 = (size_t)(v.lo[1] - alo1) * anx + (v.lo[0] - alo0);
  const int per = (cl.n + kGroups - 1) / kGroups;
  TMK_CU(cudaEventRecord(L->xfer_ev[0], 0));
  TMK_CU(cudaStreamWaitEvent(L->xfer, L->xfer_ev[0], 0));
  for (int g = 0, k0 = 0; k0 < cl.n; ++g, k0 += per) {
    tmk::CompList part{0, {}};
    for (int k = k0; k < cl.n && k < k0 + per; ++k) part.c[part.n++] = cl.c[k];
    if (in) {
      // whole rows, ghost columns included, as one contiguous block per
      // component (the staging buffer is scratch; strided copies ran slower)
      for (int k = 0; k < part.n; ++k) {
        const size_t o = (size_t)part.c[k] * anx * any + (size_t)(v.lo[1] - alo1) * anx;
        TMK_CU(cudaMemcpyAsync(L->stage + o, in + o, rows * pitch, cudaMemcpyHostToDevice, L->xfer));
      }
      TMK_CU(cudaEventRecord(L->xfer_ev[g], L->xfer));
      TMK_CU(cudaStreamWaitEvent(0, L->xfer_ev[g], 0));
      TMK_CU(tmk::copy_valid_comps(L->stage, (float*)lp.U[L->parity], alo0, alo1, anx, any, v.lo[0], v.lo[1],
                                   v.hi[0], v.hi[1], part, 0));
    } else {
      TMK_CU(tmk::copy_valid_comps((const float*)lp.U[L->parity], L->stage, alo0, alo1, anx, any, v.lo[0],
                                   v.lo[1], v.hi[0], v.hi[1], part, 0));
      TMK_CU(cudaEventRecord(L->xfer_ev[g], 0));
      TMK_CU(cudaStreamWaitEvent(L->xfer, L->xfer_ev[g], 0));
      for (int k = 0; k < part.n; ++k) {
        const size_t o = (size_t)part.c[k] * anx * any + o0;
        TMK_CU(cudaMemcpy2DAsync(out + o, pitch, L->stage + o, pitch, width, rows, cudaMemcpyDeviceToHost, L->xfer));
      }
    }
  }
  return TMK_OK;
}

// U of put/take.  Mixed form: a pinned host FAB moves through the staging
// buffer by the copy engines (valid_copy_pinned), a device FAB is read or
// written in place by the copy kernel, other host memory is staged through
// the level's FP64 staging buffer whole.  FP64 form: one strided copy per
// component.
tmk_status valid_copy(tmk_level_s* L, int p, const double* in, double* out, bool host) {
  LevelPatch& lp = L->patches[p];
  const int alo0 = lp.alloc.lo[0], alo1 = lp.alloc.lo[1];
  const int anx = lp.alloc.hi[0] - alo0 + 1, any = lp.alloc.hi[1] - alo1 + 1;
  const size_t count = (size_t)TMK_NCOMP * anx * any;
  const tmk_box& v = lp.valid;
  const tmk::CompList cl = step_comps(L);
  if (L->prec == TMK_PREC_MIXED && host && mapped_host(in ? (const void*)in : (const void*)out))
    return valid_copy_pinned(L, lp, in, out, cl);
  if (L->prec != TMK_PREC_MIXED) {
    const size_t pitch = (size_t)anx * sizeof(double);
    const size_t o0 = (size_t)(v.lo[1] - alo1) * anx + (v.lo[0] - alo0);
    for (int k = 0; k < cl.n; ++k) {
      const size_t o = (size_t)cl.c[k] * anx * any + o0;
      double* dev = (double*)lp.U[L->parity] + o;
      if (in) TMK_CU(cudaMemcpy2D(dev, pitch, in + o, pitch, (size_t)(v.hi[0] - v.lo[0] + 1) * sizeof(double),
                                  v.hi[1] - v.lo[1] + 1, cudaMemcpyDefault));
      else TMK_CU(cudaMemcpy2D(out + o, pitch, dev, pitch, (size_t)(v.hi[0] - v.lo[0] + 1) * sizeof(double),
                               v.hi[1] - v.lo[1] + 1, cudaMemcpyDefault));
    }
    return TMK_OK;
  }
  if (in) {                         // put: into the buffer the next step reads
    const double* src = host ? (const double*)mapped_host(in) : in;
    if (!src) {
      TMK_CU(cudaMemcpy(L->stage, in, count * sizeof(double), cudaMemcpyHostToDevice));
      src = L->stage;
    }
    TMK_CU(tmk::copy_valid_comps(src, (float*)lp.U[L->parity], alo0, alo1, anx, any, v.lo[0], v.lo[1], v.hi[0],
                                 v.hi[1], cl, 0));
  } else {                          // take: from the buffer the last step wrote
    double* dst = host ? (double*)mapped_host(out) : out;
    if (!dst) TMK_CU(cudaMemcpy(L->stage, out, count * sizeof(double), cudaMemcpyHostToDevice));
    TMK_CU(tmk::copy_valid_comps((const float*)lp.U[L->parity], dst ? dst : L->stage, alo0, alo1, anx, any, v.lo[0],
                                 v.lo[1], v.hi[0], v.hi[1], cl, 0));
    if (!dst) TMK_CU(cudaMemcpy(out, L->stage, count * sizeof(double), cudaMemcpyDeviceToHost));
  }
  return TMK_OK;
}

}  // namespace

extern "C" tmk_status tmk_level_put_valid(tmk_level* L, int p, const double* U, const double* B, int host) {
  if (!L || p < 0 || p >= (int)L->patches.size() || !U) return TMK_ERR_BAD_DESC;
  LevelPatch& lp = L->patches[p];
  if (lp.fault && !B) return TMK_ERR_BAD_DESC;
  tmk_status st = valid_copy(L, p, U, nullptr, host != 0);
  if (st != TMK_OK) return st;
  if (lp.fault)
    TMK_CU(cudaMemcpy(lp.B, B, (size_t)L->ctx->nb * lp.bnx * sizeof(double),
                      host ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice));
  TMK_CU(cudaDeviceSynchronize());
  return TMK_OK;
}

extern "C" tmk_status tmk_level_take_valid(tmk_level* L, int p, double* U, double* B, int host) {
  if (!L || p < 0 || p >= (int)L->patches.size() || !U) return TMK_ERR_BAD_DESC;
  LevelPatch& lp = L->patches[p];
  TMK_CU(cudaDeviceSynchronize());
  tmk_status st = valid_copy(L, p, nullptr, U, host != 0);
  if (st != TMK_OK) return st;
  if (B && lp.fault)
    TMK_CU(cudaMemcpy(B, lp.B, (size_t)L->ctx->nb * lp.bnx * sizeof(double),
                      host ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice));
  TMK_CU(cudaDeviceSynchronize());
  return TMK_OK;
}

namespace {

// The kernels of one level step after the coarse-fine fill.  Marching form:
// the in-plane kernel, then the fault kernel (scheduled as in-plane CTAs
// retire, reading only the step's input state), then the antiplane kernel
// beside it, then row 0 of the fault patches, which alone needs the fault
// results.  With the tuning's fault_first the fault kernel comes first and the
// in-plane kernel is its programmatic dependent, so that the fault kernel's
// CTAs run beside the in-plane ones.  With per-launch timing the fault kernel
// runs first and alone.
template <typename Real>
tmk_status step_kernels(tmk_level_s* L, int par, double time, double dt, cudaEvent_t* ev, cudaStream_t s) {
  tmk_context* c = L->ctx;
  const PatchDev<Real>* pd = (const PatchDev<Real>*)L->dpatch[par];
  TMK_CU(tmk::Launch<Real>::exchange(pd, L->dcopies, L->ncopies, 0, TMK_NCOMP, s));
  TMK_CU(tmk::bexchange(L->dbptr, L->dblo, L->dbnx, L->dbcopies, L->nbcopies, c->nb, s));
  if (ev) TMK_CU(cudaEventRecord(ev[1], s));
  if (!L->march) {
    TMK_CU(tmk::Launch<Real>::fault(pd, L->dfault, L->nfault, L->max_faces, L->dparams, time, c->dstatus, false, L->tune.fault_seg, s));
    if (ev) TMK_CU(cudaEventRecord(ev[2], s));
    TMK_CU(tmk::Launch<Real>::volume(pd, L->dtiles, L->ntiles, L->dparams, s));
    return TMK_OK;
  }
  tmk::MarchConst<Real> mc;
  mc.load(c->hp, dt, L->dx);
  mc.stash[0] = L->stash[0];
  mc.stash[1] = L->stash[1];
  mc.caps[0] = L->dmcap[0];
  mc.caps[1] = L->dmcap[1];
  mc.plastic = c->scheme.plasticity && L->tune.plastic_fused;
  if (mc.plastic) {
    // plastic level with the fused return: the in-plane kernel applies the
    // plastic return to each cell it stores, so it runs after the antiplane
    // kernel (its programmatic dependent, which waits for it before it
    // stores).  The fault kernel, which reads only the step's input, runs on a
    // side stream beside both and is joined before the fault rows are finished
    // (with per-launch timing it runs first and alone).
    const bool fork = L->nfault && !ev;
    if (fork) {
      if (!L->side) {
        TMK_CU(cudaStreamCreateWithFlags(&L->side, cudaStreamNonBlocking));
        TMK_CU(cudaEventCreateWithFlags(&L->fork_ev, cudaEventDisableTiming));
        TMK_CU(cudaEventCreateWithFlags(&L->join_ev, cudaEventDisableTiming));
      }
      TMK_CU(cudaEventRecord(L->fork_ev, s));
      TMK_CU(cudaStreamWaitEvent(L->side, L->fork_ev, 0));
      TMK_CU(tmk::Launch<Real>::fault(pd, L->dfault, L->nfault, L->max_faces, L->dparams, time, c->dstatus, false,
                                      L->tune.fault_seg, L->side));
      TMK_CU(cudaEventRecord(L->join_ev, L->side));
    } else {
      TMK_CU(tmk::Launch<Real>::fault(pd, L->dfault, L->nfault, L->max_faces, L->dparams, time, c->dstatus, false,
                                      L->tune.fault_seg, s));
      if (ev) TMK_CU(cudaEventRecord(ev[2], s));
    }
    TMK_CU(tmk::Launch<Real>::march(1, pd, L->ditems[1], L->nitems[1], mc, false, s));
    TMK_CU(tmk::Launch<Real>::march(0, pd, L->ditems[0], L->nitems[0], mc, !ev, s));
    if (fork) TMK_CU(cudaStreamWaitEvent(s, L->join_ev, 0));
    TMK_CU(tmk::Launch<Real>::march_fault_rows(pd, nullptr, 0, L->dfrows[1], L->nfrows[1], mc, s));
    TMK_CU(tmk::Launch<Real>::march_fault_rows(pd, L->dfrows[0], L->nfrows[0], nullptr, 0, mc, s));
    return TMK_OK;
  }
  if (ev) {
    TMK_CU(tmk::Launch<Real>::fault(pd, L->dfault, L->nfault, L->max_faces, L->dparams, time, c->dstatus, false, L->tune.fault_seg, s));
    TMK_CU(cudaEventRecord(ev[2], s));
    TMK_CU(tmk::Launch<Real>::march(0, pd, L->ditems[0], L->nitems[0], mc, false, s));
    TMK_CU(tmk::Launch<Real>::march(1, pd, L->ditems[1], L->nitems[1], mc, true, s));
  } else if (L->tune.fault_first && L->nfault) {
    TMK_CU(tmk::Launch<Real>::fault(pd, L->dfault, L->nfault, L->max_faces, L->dparams, time, c->dstatus, false, L->tune.fault_seg, s));
    TMK_CU(tmk::Launch<Real>::march(0, pd, L->ditems[0], L->nitems[0], mc, true, s));
    TMK_CU(tmk::Launch<Real>::march(1, pd, L->ditems[1], L->nitems[1], mc, true, s));
  } else {
    TMK_CU(tmk::Launch<Real>::march(0, pd, L->ditems[0], L->nitems[0], mc, false, s));
    TMK_CU(tmk::Launch<Real>::fault(pd, L->dfault, L->nfault, L->max_faces, L->dparams, time, c->dstatus, true, L->tune.fault_seg, s));
    TMK_CU(tmk::Launch<Real>::march(1, pd, L->ditems[1], L->nitems[1], mc, true, s));
  }
  TMK_CU(tmk::Launch<Real>::march_fault_rows(pd, L->dfrows[0], L->nfrows[0], L->dfrows[1], L->nfrows[1], mc, s));
  // the plastic return as a pass over the level (PLASTICCORRECTION after the update)
  if (c->scheme.plasticity) TMK_CU(tmk::Launch<Real>::plastic(pd, L->dtiles, L->ntiles, L->dparams, s));
  return TMK_OK;
}

}  // namespace

extern "C" tmk_status tmk_level_step(tmk_level* L, double time, double dt, void* stream, double* dt_new) {
  if (!L) return TMK_ERR_BAD_DESC;
  if (L->coarser) return TMK_ERR_BAD_DESC;   // a level with a coarser level needs the coarse times
  return tmk_level_step_cf(L, time, dt, 0.0, 0.0, stream, dt_new);
}

extern "C" tmk_status tmk_level_step_cf(tmk_level* L, double time, double dt, double t_coarse_old,
                                        double t_coarse_new, void* stream, double* dt_new) {
  if (!L || !(dt > 0)) return TMK_ERR_BAD_DESC;
  cudaStream_t s = (cudaStream_t)stream;
  tmk_context* c = L->ctx;
  if (dt != L->cur_dt) {
    L->cur_dt = dt;
    if (upload_patchdev(L, s) != TMK_OK) return TMK_ERR_CUDA;
  }
  const int par = L->parity;
  cudaEvent_t* ev = nullptr;
  if (L->prof_on && L->prof_n < L->prof_max) ev = &L->ev[4 * (size_t)L->prof_n++];
  if (ev) TMK_CU(cudaEventRecord(ev[0], s));
  // fault data at the start of the step (for a finer level's time interpolation)
  // and the coarse-fine ghost fill; the fill writes only ghosts that no patch
  // of this level covers, so it is independent of the same-level exchange
  tmk_status st = amr_pre_step(L, time, dt, t_coarse_old, t_coarse_new, s);
  if (st != TMK_OK) return st;
  st = L->prec == TMK_PREC_MIXED ? step_kernels<float>(L, par, time, dt, ev, s)
                                 : step_kernels<double>(L, par, time, dt, ev, s);
  if (st != TMK_OK) return st;
  // flux-register increments from the captured faces
  st = amr_post_step(L, dt, s);
  if (st != TMK_OK) return st;
  if (ev) TMK_CU(cudaEventRecord(ev[3], s));
  L->parity = 1 - par;
  // postTimeStep's station records; a level with a finer level records after
  // the finer substeps, reflux and average-down (the hierarchy step does it)
  if (L->stations && !L->finer) {
    st = tmk_stations_record(L->stations, time + dt, s);
    if (st != TMK_OK) return st;
  }
  if (dt_new) *dt_new = L->dx / std::max(c->hp.cs, c->hp.cp);
  return TMK_OK;
}

extern "C" tmk_status tmk_level_profile(tmk_level* L, int enable, int max_steps) {
  if (!L || (enable && max_steps <= 0)) return TMK_ERR_BAD_DESC;
  if (!enable) { L->prof_on = 0; return TMK_OK; }
  TMK_CU(cudaDeviceSynchronize());
  const size_t need = 4 * (size_t)max_steps;
  while (L->ev.size() < need) {
    cudaEvent_t e;
    TMK_CU(cudaEventCreate(&e));
    L->ev.push_back(e);
  }
  L->prof_on = 1; L->prof_max = max_steps; L->prof_n = 0;
  return TMK_OK;
}

extern "C" tmk_status tmk_level_profile_read(tmk_level* L, double out[4], int* nsteps) {
  if (!L || !out) return TMK_ERR_BAD_DESC;
  TMK_CU(cudaDeviceSynchronize());
  double acc[4] = {0, 0, 0, 0};
  for (int k = 0; k < L->prof_n; ++k) {
    cudaEvent_t* e = &L->ev[4 * (size_t)k];
    float a, b, cc, d;
    TMK_CU(cudaEventElapsedTime(&a, e[0], e[1]));
    TMK_CU(cudaEventElapsedTime(&b, e[1], e[2]));
    TMK_CU(cudaEventElapsedTime(&cc, e[2], e[3]));
    TMK_CU(cudaEventElapsedTime(&d, e[0], e[3]));
    acc[0] += a; acc[1] += b; acc[2] += cc; acc[3] += d;
  }
  for (int k = 0; k < 4; ++k) out[k] = L->prof_n ? acc[k] / L->prof_n : 0.0;
  if (nsteps) *nsteps = L->prof_n;
  return TMK_OK;
}

// ------------------------------------------------------------------ tuning
extern "C" tmk_status tmk_level_get_tuning(const tmk_level* L, tmk_tuning* out) {
  if (!L || !out) return TMK_ERR_BAD_DESC;
  *out = L->tune;
  return TMK_OK;
}

extern "C" tmk_status tmk_level_set_tuning(tmk_level* L, const tmk_tuning* t) {
  if (!L || !t || !tuning_ok(L, *t) || L->graphs) return TMK_ERR_BAD_DESC;
  TMK_CU(cudaDeviceSynchronize());
  L->tune = *t;
  if (L->march_allowed) {
    tmk_status st = build_march_lists(L);
    if (st != TMK_OK) return st;
  }
  L->march = L->march_allowed && t->volume_kernel == TMK_VOLUME_MARCH;
  if (L->coarser || L->finer) return tmk_host::rebuild_captures(L);
  TMK_CU(cudaDeviceSynchronize());
  return TMK_OK;
}

namespace {

// milliseconds per step of `steps` level steps after 2 untimed ones
tmk_status time_steps(tmk_level_s* L, double time, double dt, int steps, cudaStream_t s, cudaEvent_t e0,
                      cudaEvent_t e1, double* ms) {
  for (int k = 0; k < 2; ++k) {
    tmk_status st = tmk_level_step(L, time + k * dt, dt, s, nullptr);
    if (st != TMK_OK) return st;
  }
  TMK_CU(cudaEventRecord(e0, s));
  for (int k = 0; k < steps; ++k) {
    tmk_status st = tmk_level_step(L, time + (k + 2) * dt, dt, s, nullptr);
    if (st != TMK_OK) return st;
  }
  TMK_CU(cudaEventRecord(e1, s));
  TMK_CU(cudaEventSynchronize(e1));
  float f = 0.f;
  TMK_CU(cudaEventElapsedTime(&f, e0, e1));
  *ms = f / steps;
  return TMK_OK;
}

}  // namespace

// Candidate tunings of a level for the autotuners: every combination of the
// marching choices (waves per group, shortest run, fault displacement, the
// fault kernel's place in the step, on a plastic level the fused or separate
// plastic return) and both fault-kernel variants, plus the
// tile kernel; `reduced` leaves out the
// shortest runs of 8 rows (the hierarchy autotuner times whole coarse steps).
std::vector<tmk_tuning> tmk_host::tuning_candidates(const tmk_level_s* L, bool reduced) {
  std::vector<tmk_tuning> out;
  tmk_tuning t = default_tuning(L->march_allowed);
  for (int seg : {tmk::FAULT_SEG, tmk::FAULT_SEG_SMALL}) {
    t.fault_seg = seg;
    if (L->march_allowed) {
      t.volume_kernel = TMK_VOLUME_MARCH;
      for (int w0 : {1, 2})
        for (int w1 : {1, 2})
          for (int run : {8, 16, 32}) {
            if (reduced && run == 8) continue;
            for (int disp : {0, 1, 2})
              for (int first : {0, 1})
                for (int fused : {0, 1}) {
                  if (first && disp == 2) continue;
                  // the fused return fixes the kernels' order: fault_first and the
                  // displacement do not apply
                  if (fused && (!L->ctx->scheme.plasticity || first || disp)) continue;
                  t.march_waves[0] = w0; t.march_waves[1] = w1; t.min_run = run; t.fault_displace = disp;
                  t.fault_first = first;
                  t.plastic_fused = fused;
                  out.push_back(t);
                }
          }
    }
    tmk_tuning tt = default_tuning(L->march_allowed);
    tt.volume_kernel = TMK_VOLUME_TILE;
    tt.fault_seg = seg;
    out.push_back(tt);
  }
  return out;
}

namespace {
}  // namespace

extern "C" tmk_status tmk_level_autotune(tmk_level* L, double time, double dt, int steps, void* stream,
                                         tmk_tuning* best, double* ms_per_step) {
  if (!L || !(dt > 0) || steps < 1) return TMK_ERR_BAD_DESC;
  if (L->coarser || L->finer || L->graphs || L->prof_on) return TMK_ERR_BAD_DESC;
  cudaStream_t s = (cudaStream_t)stream;
  TMK_CU(cudaDeviceSynchronize());
  LevelSnapshot snap;
  tmk_status st = snap.save(L);
  if (st != TMK_OK) return st;
  const tmk_tuning t0 = L->tune;
  cudaEvent_t e0, e1;
  TMK_CU(cudaEventCreate(&e0));
  TMK_CU(cudaEventCreate(&e1));
  // every candidate once, then the four fastest twice more (mean of three)
  std::vector<tmk_tuning> cand = tuning_candidates(L, false);
  std::vector<std::pair<double, int>> timed;
  for (size_t k = 0; k < cand.size() && st == TMK_OK; ++k) {
    double ms = 0;
    if ((st = tmk_level_set_tuning(L, &cand[k])) != TMK_OK) break;
    if ((st = snap.restore(L)) != TMK_OK) break;
    if ((st = time_steps(L, time, dt, steps, s, e0, e1, &ms)) != TMK_OK) break;
    timed.push_back({ms, (int)k});
  }
  std::sort(timed.begin(), timed.end());
  const size_t top = std::min<size_t>(4, timed.size());
  for (size_t r = 0; r < 2 && st == TMK_OK; ++r)
    for (size_t q = 0; q < top && st == TMK_OK; ++q) {
      double ms = 0;
      if ((st = tmk_level_set_tuning(L, &cand[timed[q].second])) != TMK_OK) break;
      if ((st = snap.restore(L)) != TMK_OK) break;
      if ((st = time_steps(L, time, dt, steps, s, e0, e1, &ms)) != TMK_OK) break;
      timed[q].first += ms;
    }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  tmk_tuning pick = t0;
  double pick_ms = 0.0;
  if (st == TMK_OK && top) {
    size_t b = 0;
    for (size_t q = 1; q < top; ++q) if (timed[q].first < timed[b].first) b = q;
    pick = cand[timed[b].second];
    pick_ms = timed[b].first / 3.0;
  }
  tmk_status st2 = tmk_level_set_tuning(L, &pick);
  tmk_status st3 = snap.restore(L);
  if (st == TMK_OK) st = st2 != TMK_OK ? st2 : st3;
  if (st == TMK_OK) {
    if (best) *best = pick;
    if (ms_per_step) *ms_per_step = pick_ms;
  }
  return st;
}

extern "C" int tmk_level_launches_per_step(const tmk_level* L) {
  if (!L) return 0;
  // marching form: the two groups' kernels, the fault-row finisher (two
  // launches with the fused plastic return) and the plastic pass
  const bool plastic = L->ctx->scheme.plasticity != 0, fused = plastic && L->tune.plastic_fused;
  const int frows = fused ? (L->nfrows[0] ? 1 : 0) + (L->nfrows[1] ? 1 : 0) : (L->nfrows[0] + L->nfrows[1] ? 1 : 0);
  const int vol = L->march ? (L->nitems[0] ? 1 : 0) + (L->nitems[1] ? 1 : 0) + frows +
                                 (plastic && !fused && L->ntiles ? 1 : 0)
                           : (L->ntiles ? 1 : 0);
  return (L->ncopies ? 1 : 0) + (L->nbcopies ? 1 : 0) + (L->nfault ? 1 : 0) + vol + amr_launches(L);
}

extern "C" tmk_status tmk_level_status(tmk_level* L, long long info[3]) {
  if (!L || !info) return TMK_ERR_BAD_DESC;
  DevStatus h;
  TMK_CU(cudaDeviceSynchronize());
  TMK_CU(cudaMemcpy(&h, L->ctx->dstatus, sizeof(h), cudaMemcpyDeviceToHost));
  TMK_CU(cudaMemset(L->ctx->dstatus, 0, sizeof(DevStatus)));
  info[0] = h.code; info[1] = h.first_index; info[2] = (long long)h.newton_maxed;
  return h.code == 0 ? TMK_OK : (tmk_status)h.code;
}

// Read-only view of a context for other translation units of this library.
namespace tmk {
struct CtxView {
  const DevParams* dp;
  DevStatus* st;
  int fault_law;
  int nb;
  double max_speed;
};
CtxView context_view(const tmk_context* c) {
  CtxView v;
  v.dp = c->dp; v.st = c->dstatus; v.fault_law = c->scheme.fault_law; v.nb = c->nb;
  v.max_speed = std::max(c->hp.cs, c->hp.cp);
  return v;
}
}  // namespace tmk
