// Device-resident level of a CH_SPACEDIM == 3 build: the patches' FP64 state
// and fault-data FABs, the same-level ghost exchange between them
// (LevelData::exchange, as LinElastLevelGodunov::step calls it before the
// patch loop, srcLinElast/LinElastLevelGodunov.cpp:225-283) and the step: the
// exchange, the batched 3-D patch loop of tmk_patches_update_state_3d and,
// on plastic schemes, the plastic correction of every patch
// (LinElastLevelGodunov::plasticUpdate, :643-667).
#include <algorithm>
#include <cstring>
#include <vector>

#include "tmk_internal.h"

namespace {

// One rectangular copy of the exchange: components [0, ncomp) of the cells of
// region (lo, n) from the FAB over (slo, sn) to the FAB over (dlo, dn), both
// component-major, x fastest.
struct Copy3 {
  const double* src;
  double* dst;
  int slo[3], sn[3];
  int dlo[3], dn[3];
  int lo[3], n[3];
  int ncomp;
};

// Element e of a copy is (component, cell) with x fastest; the host keeps
// every copy's element count below 2^31, so the index splits in 32-bit
// unsigned divisions.
__global__ void exchange3_kernel(const Copy3* __restrict__ copies) {
  const Copy3 c = copies[blockIdx.y];
  const unsigned n0 = (unsigned)c.n[0], n1 = (unsigned)c.n[1];
  const unsigned cells = n0 * n1 * (unsigned)c.n[2];
  const unsigned total = cells * (unsigned)c.ncomp;
  const long long scs = (long long)c.sn[0] * c.sn[1] * c.sn[2];
  const long long dcs = (long long)c.dn[0] * c.dn[1] * c.dn[2];
  for (unsigned e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
    const unsigned comp = e / cells, r = e - comp * cells;
    const unsigned q = r / n0, k = q / n1;
    const int x = c.lo[0] + (int)(r - q * n0), y = c.lo[1] + (int)(q - k * n1), z = c.lo[2] + (int)k;
    const long long so = comp * scs + ((long long)(z - c.slo[2]) * c.sn[1] + (y - c.slo[1])) * c.sn[0] + (x - c.slo[0]);
    const long long dof = comp * dcs + ((long long)(z - c.dlo[2]) * c.dn[1] + (y - c.dlo[1])) * c.dn[0] + (x - c.dlo[0]);
    c.dst[dof] = c.src[so];
  }
}

bool box3_ok(const tmk_box3& b) { return b.lo[0] <= b.hi[0] && b.lo[1] <= b.hi[1] && b.lo[2] <= b.hi[2]; }
tmk_box3 box3_isect(const tmk_box3& a, const tmk_box3& b) {
  tmk_box3 r;
  for (int d = 0; d < 3; ++d) {
    r.lo[d] = std::max(a.lo[d], b.lo[d]);
    r.hi[d] = std::min(a.hi[d], b.hi[d]);
  }
  return r;
}
bool box3_contains(const tmk_box3& a, const tmk_box3& b) {
  for (int d = 0; d < 3; ++d)
    if (b.lo[d] < a.lo[d] || b.hi[d] > a.hi[d]) return false;
  return true;
}
size_t fab_count(const tmk_fab3& f) {
  return (size_t)f.ncomp * (f.hi[0] - f.lo[0] + 1) * (f.hi[1] - f.lo[1] + 1) * (f.hi[2] - f.lo[2] + 1);
}
Copy3 make_copy(const tmk_fab3& src, const tmk_fab3& dst, const tmk_box3& g) {
  Copy3 c;
  c.src = src.data;
  c.dst = dst.data;
  for (int d = 0; d < 3; ++d) {
    c.slo[d] = src.lo[d]; c.sn[d] = src.hi[d] - src.lo[d] + 1;
    c.dlo[d] = dst.lo[d]; c.dn[d] = dst.hi[d] - dst.lo[d] + 1;
    c.lo[d] = g.lo[d]; c.n[d] = g.hi[d] - g.lo[d] + 1;
  }
  c.ncomp = src.ncomp;
  return c;
}

}  // namespace

struct tmk_level3d_s {
  tmk_context* ctx = nullptr;
  tmk_box3 domain{};
  double dx = 0.0;
  std::vector<tmk_box3> valid;
  std::vector<tmk_fab3> U;       // over grow(valid, TMK_NGHOST)
  std::vector<tmk_fab3> B;       // fault patches: over grow(valid, TMK_NGHOST) in x, z on the y-lo plane
  bool any_fault = false;
  Copy3* dcopies = nullptr;      // state copies, then fault-data copies
  int ncopies = 0;
  std::vector<void*> allocs;
};

extern "C" void tmk_level3d_destroy(tmk_level3d* L) {
  if (!L) return;
  cudaDeviceSynchronize();
  for (void* p : L->allocs) cudaFree(p);
  delete L;
}

extern "C" tmk_status tmk_level3d_create(tmk_context* ctx, const tmk_box3* domain, double dx, int npatch,
                                         const tmk_box3* boxes, tmk_level3d** out) {
  if (!ctx || !domain || !boxes || !out || npatch < 1 || !(dx > 0) || !box3_ok(*domain)) return TMK_ERR_BAD_DESC;
  *out = nullptr;
  for (int p = 0; p < npatch; ++p) {
    if (!box3_ok(boxes[p]) || !box3_contains(*domain, boxes[p])) return TMK_ERR_BAD_DESC;
    for (int q = 0; q < p; ++q)
      if (box3_ok(box3_isect(boxes[p], boxes[q]))) return TMK_ERR_BAD_DESC;   // valid boxes overlap
  }
  tmk_level3d* L = new tmk_level3d;
  auto fail = [&](tmk_status st) { tmk_level3d_destroy(L); return st; };
  L->ctx = ctx;
  L->domain = *domain;
  L->dx = dx;
  L->valid.assign(boxes, boxes + npatch);
  const bool law = ctx->scheme.fault_law != TMK_FAULT_NONE;
  const int g = TMK_NGHOST;
  for (int p = 0; p < npatch; ++p) {
    tmk_fab3 u{};
    for (int d = 0; d < 3; ++d) { u.lo[d] = boxes[p].lo[d] - g; u.hi[d] = boxes[p].hi[d] + g; }
    u.ncomp = TMK_NCOMP;
    if (cudaMalloc(&u.data, fab_count(u) * sizeof(double)) != cudaSuccess) return fail(TMK_ERR_ALLOC);
    L->allocs.push_back(u.data);
    L->U.push_back(u);
    tmk_fab3 b{};
    if (law && boxes[p].lo[1] == domain->lo[1]) {
      b = u;
      b.lo[1] = b.hi[1] = domain->lo[1];
      b.ncomp = ctx->nb;
      if (cudaMalloc(&b.data, fab_count(b) * sizeof(double)) != cudaSuccess) return fail(TMK_ERR_ALLOC);
      L->allocs.push_back(b.data);
      L->any_fault = true;
    }
    L->B.push_back(b);
  }
  // exchange lists: the ghost cells of p inside the domain that the valid box
  // of q covers, as far as the step reads them (the state over grow(valid, 3),
  // the fault data over grow(valid, 1) in x and z: tmk_patch_update_state_3d);
  // the ghost layers beyond are left as they are
  std::vector<Copy3> copies;
  auto grown = [](tmk_box3 b, int n, bool y) {
    for (int d = 0; d < 3; ++d)
      if (d != 1 || y) { b.lo[d] -= n; b.hi[d] += n; }
    return b;
  };
  for (int p = 0; p < npatch; ++p)
    for (int q = 0; q < npatch; ++q) {
      if (p == q) continue;
      const tmk_box3 gu = box3_isect(box3_isect(grown(boxes[p], 3, true), boxes[q]), *domain);
      if (box3_ok(gu)) copies.push_back(make_copy(L->U[q], L->U[p], gu));
    }
  for (int p = 0; p < npatch; ++p)
    for (int q = 0; q < npatch; ++q) {
      if (p == q || !L->B[p].data || !L->B[q].data) continue;
      tmk_box3 reach = grown(boxes[p], 1, false), vq = boxes[q];   // on the plane
      reach.lo[1] = reach.hi[1] = vq.lo[1] = vq.hi[1] = domain->lo[1];
      const tmk_box3 gb = box3_isect(box3_isect(reach, vq), *domain);
      if (box3_ok(gb)) copies.push_back(make_copy(L->B[q], L->B[p], gb));
    }
  for (const Copy3& c : copies)
    if ((long long)c.n[0] * c.n[1] * c.n[2] * c.ncomp >= (1LL << 31)) return fail(TMK_ERR_BAD_DESC);
  L->ncopies = (int)copies.size();
  if (L->ncopies) {
    if (cudaMalloc(&L->dcopies, copies.size() * sizeof(Copy3)) != cudaSuccess) return fail(TMK_ERR_ALLOC);
    L->allocs.push_back(L->dcopies);
    if (cudaMemcpy(L->dcopies, copies.data(), copies.size() * sizeof(Copy3), cudaMemcpyHostToDevice) != cudaSuccess)
      return fail(TMK_ERR_CUDA);
  }
  *out = L;
  return TMK_OK;
}

namespace {

tmk_status patch_fabs(const tmk_level3d* L, int p, const tmk_fab3** u, const tmk_fab3** b) {
  if (!L || p < 0 || p >= (int)L->U.size()) return TMK_ERR_BAD_DESC;
  *u = &L->U[p];
  *b = L->B[p].data ? &L->B[p] : nullptr;
  return TMK_OK;
}

}  // namespace

extern "C" tmk_status tmk_level3d_set_patch(tmk_level3d* L, int p, const double* U, const double* B, int host) {
  const tmk_fab3 *u, *b;
  tmk_status st = patch_fabs(L, p, &u, &b);
  if (st != TMK_OK) return st;
  if (!U || (b && !B)) return TMK_ERR_BAD_DESC;
  const cudaMemcpyKind kind = host ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
  TMK_CU(cudaMemcpy(u->data, U, fab_count(*u) * sizeof(double), kind));
  if (b) TMK_CU(cudaMemcpy(b->data, B, fab_count(*b) * sizeof(double), kind));
  return TMK_OK;
}

extern "C" tmk_status tmk_level3d_get_patch(tmk_level3d* L, int p, double* U, double* B, int host) {
  const tmk_fab3 *u, *b;
  tmk_status st = patch_fabs(L, p, &u, &b);
  if (st != TMK_OK) return st;
  if (!U) return TMK_ERR_BAD_DESC;
  TMK_CU(cudaDeviceSynchronize());
  const cudaMemcpyKind kind = host ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
  TMK_CU(cudaMemcpy(U, u->data, fab_count(*u) * sizeof(double), kind));
  if (b && B) TMK_CU(cudaMemcpy(B, b->data, fab_count(*b) * sizeof(double), kind));
  return TMK_OK;
}

extern "C" tmk_status tmk_level3d_patch_fabs(const tmk_level3d* L, int p, tmk_fab3* U, tmk_fab3* B) {
  const tmk_fab3 *u, *b;
  tmk_status st = patch_fabs(L, p, &u, &b);
  if (st != TMK_OK) return st;
  if (U) *U = *u;
  if (B) {
    if (b) *B = *b;
    else *B = tmk_fab3{};
  }
  return TMK_OK;
}

extern "C" tmk_status tmk_level3d_exchange(tmk_level3d* L, void* stream) {
  if (!L) return TMK_ERR_BAD_DESC;
  const cudaStream_t s = (cudaStream_t)stream;
  for (int c0 = 0; c0 < L->ncopies; c0 += 65535) {
    const int n = std::min(65535, L->ncopies - c0);
    exchange3_kernel<<<dim3(16, n), 256, 0, s>>>(L->dcopies + c0);
    TMK_CU(cudaGetLastError());
  }
  return TMK_OK;
}

extern "C" tmk_status tmk_level3d_step(tmk_level3d* L, double time, double dt, double* max_wave_speed,
                                       void* stream) {
  if (!L || !(dt > 0)) return TMK_ERR_BAD_DESC;
  tmk_status st = tmk_level3d_exchange(L, stream);
  if (st != TMK_OK) return st;
  const int np = (int)L->U.size();
  st = tmk_patches_update_state_3d(L->ctx, np, L->U.data(), L->any_fault ? L->B.data() : nullptr, nullptr, nullptr,
                                   nullptr, L->valid.data(), &L->domain, L->dx, time, dt, max_wave_speed, stream);
  if (st != TMK_OK) return st;
  if (L->ctx->scheme.plasticity)
    for (int p = 0; p < np; ++p)
      if ((st = tmk_plastic_update_3d(L->ctx, &L->U[p], &L->valid[p], dt, stream)) != TMK_OK) return st;
  return TMK_OK;
}
