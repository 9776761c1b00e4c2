// noalloc.cu -- the density filter for callers that cannot allocate device
// memory.
//
// Some callers cannot call cudaMalloc at the point where they need the filter:
// code that runs inside an allocator-free real-time or serving loop, hosts whose
// device memory is owned by another runtime's arena (a JVM, Swift or game-engine
// host handing out pre-sized buffers), or code paths that must not touch the
// CUDA allocator once they have started.  They own their inputs and outputs
// already; what they cannot do is let the library allocate the filter's
// scratch (the per-voxel weight sums, the adjoint's scaled sensitivity, the
// stencil table, the solid mask).  tg_filter_noalloc runs the same filter
// kernels as tg_filter, with that scratch in one fixed, file-scope device array.
//
// Limits and sharing:
//  * at most kNoAllocMaxVoxels voxels and kNoAllocMaxStencil stencil entries
//    (filter radius up to 6 voxels); larger requests are rejected with TG_EINVAL;
//  * the array is a static __device__ object: every GPU that loads the library
//    holds its ~17 MB until the process exits;
//  * every call shares it, so calls whose work overlaps on the GPU (different
//    streams, or different host threads, without ordering between them) race:
//    serialise them on one stream;
//  * nothing in the scratch carries over between calls: each call rewrites every
//    entry it reads (mask, stencil, weight sums, scaled sensitivity) before
//    reading it, so no clearing is needed and a call's result does not depend
//    on the previous call's contents;
//  * every call, with the target device current, looks up the array's device
//    address with cudaGetSymbolAddress (host code cannot use the symbol itself:
//    on the host it names a stand-in, not device memory).  The first call on
//    a device may load the library's module there; make it before any stream
//    capture begins.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <string>

#include "tg_internal.h"

namespace tg {
namespace {

constexpr int64_t kNoAllocMaxVoxels = int64_t(1) << 20;  // 1,048,576 voxels
constexpr int kNoAllocMaxStencil = 1024;                // covers radius <= 6
constexpr int kMaxDevices = 64;

// Layout-identical to the stencil entries the filter kernels read (k_simp.cu).
struct NoAllocStencilEntry {
  int di, dj, dk, pad;
  double w;
};
static_assert(sizeof(NoAllocStencilEntry) == 24, "stencil entry layout");

struct NoAllocScratch {
  double hs[kNoAllocMaxVoxels];   // weight sums Hs
  double tmp[kNoAllocMaxVoxels];  // adjoint: s_e / Hs_e
  NoAllocStencilEntry st[kNoAllocMaxStencil];
  uint8_t act[kNoAllocMaxVoxels];  // solid mask
};

static __device__ __align__(256) NoAllocScratch g_noalloc_scratch;

// The array's device address in the current device's context.  Looked up on
// every call (a symbol lookup; it allocates nothing), so the address always
// belongs to the context that is current now -- also after cudaDeviceReset or a
// primary context that was torn down and created again.
NoAllocScratch* scratch_for_current_device() {
  int dev = 0;
  TG_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) raise(TG_EINVAL, "tg_filter_noalloc: device ordinal too large");
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess || p == nullptr)
    raise(TG_EDEVICE, std::string("tg_filter_noalloc: cudaGetSymbolAddress of the scratch "
                                  "array failed: ") + cudaGetErrorString(e));
  return static_cast<NoAllocScratch*>(p);
}

// Same stencil as FilterStencil::make: offsets in (dk, dj, di) ascending order
// with weight r - |d| > 0.  One thread; the host counts the entries the same way.
__global__ void k_noalloc_stencil(double radius, int R, NoAllocStencilEntry* st) {
  int q = 0;
  for (int dk = -R; dk <= R; ++dk)
    for (int dj = -R; dj <= R; ++dj)
      for (int di = -R; di <= R; ++di) {
        const double w = radius - sqrt(double(di * di + dj * dj + dk * dk));
        if (w <= 0.0) continue;
        st[q].di = di;
        st[q].dj = dj;
        st[q].dk = dk;
        st[q].pad = 0;
        st[q].w = w;
        ++q;
      }
}

__global__ void k_noalloc_mask(const uint8_t* __restrict__ tags, int64_t n, uint8_t* __restrict__ act) {
  for (int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; e < n;
       e += int64_t(gridDim.x) * blockDim.x)
    act[e] = tags == nullptr ? uint8_t(1) : uint8_t(tags[e] != 0);
}

int stencil_count(double radius, int R) {
  int q = 0;
  for (int dk = -R; dk <= R; ++dk)
    for (int dj = -R; dj <= R; ++dj)
      for (int di = -R; di <= R; ++di)
        if (radius - std::sqrt(double(di * di + dj * dj + dk * dk)) > 0.0) ++q;
  return q;
}

}  // namespace
}  // namespace tg

extern "C" int tg_filter_noalloc(int32_t nx, int32_t ny, int32_t nz, const uint8_t* d_tags,
                                 double radius, int32_t adjoint, const double* d_x, double* d_out,
                                 void* stream) {
  using namespace tg;
  try {
    if (nx < 1 || ny < 1 || nz < 1) raise(TG_EINVAL, "tg_filter_noalloc: grid dimensions must be >= 1");
    const int64_t nv = int64_t(nx) * ny * nz;
    if (nv > kNoAllocMaxVoxels)
      raise(TG_EINVAL, "tg_filter_noalloc: grid has more than 1,048,576 voxels, the fixed "
                       "scratch limit; use tg_filter");
    if (!(radius > 0.0)) raise(TG_EINVAL, "make_density_filter: radius must be > 0");
    if (radius > 6.0) raise(TG_EINVAL, "tg_filter_noalloc: radius above 6 voxels exceeds the fixed stencil limit");
    if (!d_x || !d_out) raise(TG_EINVAL, "tg_filter_noalloc: d_x and d_out must be device pointers");
    const int R = int(std::ceil(radius));
    const int ns = stencil_count(radius, R);
    if (ns > kNoAllocMaxStencil) raise(TG_EINVAL, "tg_filter_noalloc: stencil too large");
    NoAllocScratch* sc = scratch_for_current_device();
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const Grid g = Grid::make(nx, ny, nz, 1.0);
    k_noalloc_stencil<<<1, 1, 0, s>>>(radius, R, sc->st);
    TG_LAUNCH_CHECK();
    const int blocks = int(std::min<int64_t>((nv + 255) / 256, 152 * 32));
    k_noalloc_mask<<<blocks, 256, 0, s>>>(d_tags, nv, sc->act);
    TG_LAUNCH_CHECK();
    launch_weight_sum(g, sc->st, ns, sc->act, sc->hs, s);
    if (adjoint)
      launch_filter_adj(g, sc->st, ns, sc->act, sc->hs, d_x, sc->tmp, d_out, s);
    else
      launch_filter_fwd(g, sc->st, ns, sc->act, sc->hs, d_x, d_out, s);
    return TG_OK;
  } catch (const Error& e) {
    set_last_error(e.what());
    return e.code;
  }
}
