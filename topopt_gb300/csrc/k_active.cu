// k_active.cu -- the active-domain mask of the restricted trajectory solves.
//
// Reference counterparts (core/src/simp/simp.cpp):
//   active_domain_mask          :449-528   core + Load/Fixture pin, Chebyshev band
//   active_domain_escape_count  :530-556
//
// The mask is integer work on voxel bytes: a core pass over the density, three
// dilation passes (x, then y, then z; a cube of half-width `band` is the
// product of three segments, so three passes give the Chebyshev dilation
// exactly), and a pass that ANDs with the solid set and counts.  Each pass is
// one thread per voxel on a 3D grid (x the fastest axis, so every read of a
// pass is coalesced along x, including the y and z passes, whose window walks
// whole rows).  No floating-point value is combined, so the mask is the
// reference's bit for bit.  Counts are integer atomics of one warp-aggregated
// add per warp: order-independent, deterministic.
#include <cuda_runtime.h>

#include <cstdint>

#include "tg_internal.h"

namespace tg {

namespace {
constexpr int kAdThreads = 128;

__device__ __forceinline__ bool ad_solid(const uint8_t* tags, int64_t e) {
  return tags == nullptr || tags[e] != 0;
}

// m[e] = solid AND (rho > thresh OR tag Load (4) OR tag Fixture (5)).
__global__ void k_ad_core(const uint8_t* __restrict__ tags, const double* __restrict__ rho,
                          double thresh, int64_t nv, uint8_t* __restrict__ m) {
  for (int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; e < nv;
       e += int64_t(gridDim.x) * blockDim.x) {
    const uint8_t t = tags ? tags[e] : uint8_t(1);
    m[e] = uint8_t(t != 0 && (rho[e] > thresh || t == 4 || t == 5));
  }
}

// out = 1 where `in` has a set voxel on the same line of `axis` within `band`.
__global__ void k_ad_dilate(int nx, int ny, int nz, int axis, int band,
                            const uint8_t* __restrict__ in, uint8_t* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, k = blockIdx.z;
  if (i >= nx) return;
  const int64_t e = (int64_t(k) * ny + j) * nx + i;
  const int pos = axis == 0 ? i : axis == 1 ? j : k;
  const int len = axis == 0 ? nx : axis == 1 ? ny : nz;
  const int64_t stride = axis == 0 ? 1 : axis == 1 ? int64_t(nx) : int64_t(nx) * ny;
  const int lo = pos - band < 0 ? 0 : pos - band;
  const int hi = pos + band > len - 1 ? len - 1 : pos + band;
  uint8_t v = 0;
  for (int t = lo; t <= hi && !v; ++t) v = in[e + int64_t(t - pos) * stride];
  out[e] = v;
}

__device__ __forceinline__ void warp_count(bool v, unsigned long long* count) {
  const unsigned ballot = __ballot_sync(0xffffffffu, v);
  if ((threadIdx.x & 31) == 0 && ballot) atomicAdd(count, (unsigned long long)__popc(ballot));
}

// out[e] = band-set (or 1 when `t` is null: the band covers everything) AND
// solid; count += ones.  The grid-stride loop keeps whole warps in step so the
// ballot sees every lane (lanes past nv vote 0).
__global__ void k_ad_finish(const uint8_t* __restrict__ tags, const uint8_t* __restrict__ t,
                            int64_t nv, uint8_t* __restrict__ out,
                            unsigned long long* __restrict__ count) {
  const int64_t step = int64_t(gridDim.x) * blockDim.x;
  for (int64_t base = blockIdx.x * int64_t(blockDim.x); base < nv; base += step) {
    const int64_t e = base + threadIdx.x;
    bool v = false;
    if (e < nv) {
      v = (t == nullptr || t[e] != 0) && ad_solid(tags, e);
      out[e] = uint8_t(v);
    }
    warp_count(v, count);
  }
}

__global__ void k_ad_escape(const uint8_t* __restrict__ tags, const double* __restrict__ rho,
                            const uint8_t* __restrict__ prev, double thresh, int64_t nv,
                            unsigned long long* __restrict__ count) {
  const int64_t step = int64_t(gridDim.x) * blockDim.x;
  for (int64_t base = blockIdx.x * int64_t(blockDim.x); base < nv; base += step) {
    const int64_t e = base + threadIdx.x;
    const bool v = e < nv && ad_solid(tags, e) && prev[e] == 0 && rho[e] > thresh;
    warp_count(v, count);
  }
}

int ad_blocks(int64_t n) {
  const int64_t b = (n + kAdThreads - 1) / kAdThreads;
  return int(b < 152 * 16 ? (b > 0 ? b : 1) : 152 * 16);
}
}  // namespace

void launch_active_domain_mask(int nx, int ny, int nz, const uint8_t* tags, const double* rho,
                               double density_min, int band, uint8_t* out, uint8_t* tmp,
                               unsigned long long* count, cudaStream_t s) {
  const int64_t nv = int64_t(nx) * ny * nz;
  TG_CUDA(cudaMemsetAsync(count, 0, sizeof(unsigned long long), s));
  if (band <= 0) {  // off: every solid voxel
    k_ad_finish<<<ad_blocks(nv), kAdThreads, 0, s>>>(tags, nullptr, nv, out, count);
    TG_LAUNCH_CHECK();
    return;
  }
  k_ad_core<<<ad_blocks(nv), kAdThreads, 0, s>>>(tags, rho, 1.5 * density_min, nv, out);
  TG_LAUNCH_CHECK();
  const dim3 grid((nx + kAdThreads - 1) / kAdThreads, ny, nz);
  // A band past an axis' length reaches the whole line; clamping keeps the
  // window arithmetic in range.
  const int bx = band < nx ? band : nx, by = band < ny ? band : ny, bz = band < nz ? band : nz;
  k_ad_dilate<<<grid, kAdThreads, 0, s>>>(nx, ny, nz, 0, bx, out, tmp);
  TG_LAUNCH_CHECK();
  k_ad_dilate<<<grid, kAdThreads, 0, s>>>(nx, ny, nz, 1, by, tmp, out);
  TG_LAUNCH_CHECK();
  k_ad_dilate<<<grid, kAdThreads, 0, s>>>(nx, ny, nz, 2, bz, out, tmp);
  TG_LAUNCH_CHECK();
  k_ad_finish<<<ad_blocks(nv), kAdThreads, 0, s>>>(tags, tmp, nv, out, count);
  TG_LAUNCH_CHECK();
}

void launch_active_domain_escape(const uint8_t* tags, const double* rho, const uint8_t* prev,
                                 double density_min, int64_t nv, unsigned long long* count,
                                 cudaStream_t s) {
  TG_CUDA(cudaMemsetAsync(count, 0, sizeof(unsigned long long), s));
  k_ad_escape<<<ad_blocks(nv), kAdThreads, 0, s>>>(tags, rho, prev, 1.5 * density_min, nv, count);
  TG_LAUNCH_CHECK();
}

}  // namespace tg
