// FP64 instantiation (plain form).  Compiled with --fmad=false so that every
// product and sum rounds as in the reference's Fortran and the CPU oracle.
#include "tmk_launch_impl.cuh"
TMK_INSTANTIATE_LAUNCH(double, 16, 8, 256)

namespace tmk {

__global__ void plastic_fab_kernel(double* U, int alo0, int alo1, int anx, int any, int lo0, int lo1, int hi0,
                                   int hi1, const DevParams* P, double dt) {
  const int nx = hi0 - lo0 + 1, ny = hi1 - lo1 + 1;
  const size_t plane = (size_t)anx * any;
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < nx * ny; idx += gridDim.x * blockDim.x) {
    int i = lo0 + idx % nx, j = lo1 + idx / nx;
    size_t o = (size_t)(j - alo1) * anx + (i - alo0);
    for (int s = 0; s < 2; ++s) {
      double* u = U + (size_t)(11 * s) * plane + o;
      double sxx = u[3 * plane], syy = u[4 * plane], szz = u[5 * plane], sxy = u[6 * plane];
      double sxz = u[7 * plane], syz = u[8 * plane], lam = u[9 * plane], gam = u[10 * plane];
      plastic_flow<double>(*P, sxx, syy, szz, sxy, sxz, syz, lam, gam, dt);
      u[3 * plane] = sxx; u[4 * plane] = syy; u[5 * plane] = szz; u[6 * plane] = sxy;
      u[7 * plane] = sxz; u[8 * plane] = syz; u[9 * plane] = lam; u[10 * plane] = gam;
    }
  }
}

cudaError_t plastic_fab(double* U, int alo0, int alo1, int anx, int any, int lo0, int lo1, int hi0, int hi1,
                        const DevParams* P, double dt, cudaStream_t s) {
  int n = (hi0 - lo0 + 1) * (hi1 - lo1 + 1);
  if (n <= 0) return cudaSuccess;
  int blocks = (n + 255) / 256;
  if (blocks > 4096) blocks = 4096;
  plastic_fab_kernel<<<blocks, 256, 0, s>>>(U, alo0, alo1, anx, any, lo0, lo1, hi0, hi1, P, dt);
  return cudaGetLastError();
}

__global__ void copy_valid_kernel(const double* src, double* dst, int alo0, int alo1, int anx, int any, int vlo0,
                                  int vlo1, int vhi0, int vhi1, int c0, int ncomp) {
  const int nx = vhi0 - vlo0 + 1, ny = vhi1 - vlo1 + 1;
  const size_t n = (size_t)ncomp * nx * ny;
  for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += (size_t)gridDim.x * blockDim.x) {
    int c = c0 + (int)(idx / ((size_t)nx * ny)), j = vlo1 + (int)((idx / nx) % ny), i = vlo0 + (int)(idx % nx);
    size_t o = ((size_t)c * any + (j - alo1)) * anx + (i - alo0);
    dst[o] = src[o];
  }
}

cudaError_t copy_valid(const double* src, double* dst, int alo0, int alo1, int anx, int any, int vlo0, int vlo1,
                       int vhi0, int vhi1, int c0, int ncomp, cudaStream_t s) {
  size_t n = (size_t)ncomp * (vhi0 - vlo0 + 1) * (vhi1 - vlo1 + 1);
  if (n == 0) return cudaSuccess;
  size_t blocks = (n + 255) / 256;
  if (blocks > 8192) blocks = 8192;
  copy_valid_kernel<<<(unsigned)blocks, 256, 0, s>>>(src, dst, alo0, alo1, anx, any, vlo0, vlo1, vhi0, vhi1, c0, ncomp);
  return cudaGetLastError();
}

// Whole-FAB conversion or copy, four elements per thread in flight (all loads,
// then all stores).  Either side may be pinned host memory seen through its
// device address, so a set or get of a level's state crosses the host link
// once, inside this kernel, with no staging copy.
template <typename S, typename D>
__global__ void convert_kernel(const S* __restrict__ a, D* __restrict__ b, size_t n) {
  constexpr int U = 4;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  for (; i + (U - 1) * stride < n; i += U * stride) {
    S v[U];
#pragma unroll
    for (int u = 0; u < U; ++u) v[u] = a[i + u * stride];
#pragma unroll
    for (int u = 0; u < U; ++u) b[i + u * stride] = (D)v[u];
  }
  for (; i < n; i += stride) b[i] = (D)a[i];
}
template <typename S, typename D>
cudaError_t convert_launch(const S* src, D* dst, size_t n, cudaStream_t s) {
  if (!n) return cudaSuccess;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return cudaErrorUnknown;
  const size_t want = (n + 4 * 256 - 1) / (4 * 256);
  const unsigned blocks = (unsigned)std::max<size_t>(1, std::min<size_t>(want, (size_t)sms * 8));
  convert_kernel<S, D><<<blocks, 256, 0, s>>>(src, dst, n);
  return cudaGetLastError();
}
// One row of one listed component per pass of a CTA (rows of the valid box
// are contiguous runs of the FAB), four elements per thread in flight: a put
// or take of a level's state crosses the host link once, inside this kernel.
template <typename S, typename D>
__global__ void valid_comps_kernel(const S* __restrict__ a, D* __restrict__ b, int alo0, int alo1, int anx,
                                   int any, int vlo0, int vlo1, int vnx, int vny, CompList cl) {
  constexpr int U = 4;
  const int nrows = cl.n * vny;
  for (int r = blockIdx.x; r < nrows; r += gridDim.x) {
    const int c = cl.c[r / vny], j = vlo1 + r % vny;
    const size_t o = ((size_t)c * any + (j - alo1)) * anx + (vlo0 - alo0);
    int i = threadIdx.x;
    for (; i + (U - 1) * (int)blockDim.x < vnx; i += U * blockDim.x) {
      S v[U];
#pragma unroll
      for (int u = 0; u < U; ++u) v[u] = a[o + i + u * blockDim.x];
#pragma unroll
      for (int u = 0; u < U; ++u) b[o + i + u * blockDim.x] = (D)v[u];
    }
    for (; i < vnx; i += blockDim.x) b[o + i] = (D)a[o + i];
  }
}
// The same with two elements per access (16-byte host reads or writes: fewer,
// larger requests over the host link), for rows whose valid run starts on an
// even element of 16-byte aligned FABs and has even length.
template <typename S, typename D> struct Vec2;
template <> struct Vec2<double, float> { using SV = double2; using DV = float2;
  static __device__ DV cv(SV v) { return make_float2((float)v.x, (float)v.y); } };
template <> struct Vec2<float, double> { using SV = float2; using DV = double2;
  static __device__ DV cv(SV v) { return make_double2((double)v.x, (double)v.y); } };
template <> struct Vec2<double, double> { using SV = double2; using DV = double2;
  static __device__ DV cv(SV v) { return v; } };
template <typename S, typename D>
__global__ void valid_comps_kernel2(const S* __restrict__ a, D* __restrict__ b, int alo0, int alo1, int anx,
                                    int any, int vlo0, int vlo1, int vnx, int vny, CompList cl) {
  using V = Vec2<S, D>;
  constexpr int U = 4;
  const int nrows = cl.n * vny, nv = vnx / 2;
  for (int r = blockIdx.x; r < nrows; r += gridDim.x) {
    const int c = cl.c[r / vny], j = vlo1 + r % vny;
    const size_t o = ((size_t)c * any + (j - alo1)) * anx + (vlo0 - alo0);
    const typename V::SV* av = reinterpret_cast<const typename V::SV*>(a + o);
    typename V::DV* bv = reinterpret_cast<typename V::DV*>(b + o);
    int i = threadIdx.x;
    for (; i + (U - 1) * (int)blockDim.x < nv; i += U * blockDim.x) {
      typename V::SV v[U];
#pragma unroll
      for (int u = 0; u < U; ++u) v[u] = av[i + u * blockDim.x];
#pragma unroll
      for (int u = 0; u < U; ++u) bv[i + u * blockDim.x] = V::cv(v[u]);
    }
    for (; i < nv; i += blockDim.x) bv[i] = V::cv(av[i]);
  }
}
template <typename S, typename D>
cudaError_t valid_comps_launch(const S* src, D* dst, int alo0, int alo1, int anx, int any, int vlo0, int vlo1,
                               int vhi0, int vhi1, const CompList& cl, cudaStream_t s) {
  const int vnx = vhi0 - vlo0 + 1, vny = vhi1 - vlo1 + 1;
  if (vnx <= 0 || vny <= 0 || cl.n <= 0) return cudaSuccess;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return cudaErrorUnknown;
  const unsigned blocks = (unsigned)std::max(1, std::min(cl.n * vny, sms * 8));
  const bool pairs = ((uintptr_t)src % 16) == 0 && ((uintptr_t)dst % (2 * sizeof(D))) == 0 && anx % 2 == 0 &&
                     (vlo0 - alo0) % 2 == 0 && vnx % 2 == 0;
  if (pairs)
    valid_comps_kernel2<S, D><<<blocks, 256, 0, s>>>(src, dst, alo0, alo1, anx, any, vlo0, vlo1, vnx, vny, cl);
  else
    valid_comps_kernel<S, D><<<blocks, 256, 0, s>>>(src, dst, alo0, alo1, anx, any, vlo0, vlo1, vnx, vny, cl);
  return cudaGetLastError();
}
cudaError_t copy_valid_comps(const double* src, float* dst, int alo0, int alo1, int anx, int any, int vlo0, int vlo1,
                             int vhi0, int vhi1, const CompList& cl, cudaStream_t s) {
  return valid_comps_launch(src, dst, alo0, alo1, anx, any, vlo0, vlo1, vhi0, vhi1, cl, s);
}
cudaError_t copy_valid_comps(const float* src, double* dst, int alo0, int alo1, int anx, int any, int vlo0, int vlo1,
                             int vhi0, int vhi1, const CompList& cl, cudaStream_t s) {
  return valid_comps_launch(src, dst, alo0, alo1, anx, any, vlo0, vlo1, vhi0, vhi1, cl, s);
}
cudaError_t copy_valid_comps(const double* src, double* dst, int alo0, int alo1, int anx, int any, int vlo0,
                             int vlo1, int vhi0, int vhi1, const CompList& cl, cudaStream_t s) {
  return valid_comps_launch(src, dst, alo0, alo1, anx, any, vlo0, vlo1, vhi0, vhi1, cl, s);
}

cudaError_t convert_d2f(const double* src, float* dst, size_t n, cudaStream_t s) { return convert_launch(src, dst, n, s); }
cudaError_t convert_f2d(const float* src, double* dst, size_t n, cudaStream_t s) { return convert_launch(src, dst, n, s); }
cudaError_t copy_fab(const double* src, double* dst, size_t n, cudaStream_t s) { return convert_launch(src, dst, n, s); }

// Fault-row exchange: copy boundary data faces [lo0, hi0] from src to dst patch.
__global__ void bexchange_kernel(double* const* __restrict__ bptr, const int* __restrict__ blo,
                                 const int* __restrict__ bnx, const CopyDev* __restrict__ copies, int nb) {
  const CopyDev cp = copies[blockIdx.x];
  const int n = cp.hi0 - cp.lo0 + 1;
  for (int idx = threadIdx.x; idx < nb * n; idx += blockDim.x) {
    int c = idx / n, i = cp.lo0 + idx % n;
    bptr[cp.dst][(size_t)c * bnx[cp.dst] + (i - blo[cp.dst])] = bptr[cp.src][(size_t)c * bnx[cp.src] + (i - blo[cp.src])];
  }
}


cudaError_t bexchange(double* const* bptr, const int* blo, const int* bnx, const CopyDev* copies, int ncopies,
                      int nb, cudaStream_t s) {
  if (ncopies <= 0) return cudaSuccess;
  bexchange_kernel<<<ncopies, 128, 0, s>>>(bptr, blo, bnx, copies, nb);
  return cudaGetLastError();
}

}  // namespace tmk
