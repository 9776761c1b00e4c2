// k_vector.cu -- PCG vector updates and deterministic FP64 reductions.
//
// Reference counterpart: the dot products and AXPYs of mf_cg_solve and mf_mgpcg
// (core/src/fea/matfree.cpp:1006-1060, core/src/fea/multigrid.cpp:1287-1310).
// Every reduction runs on a fixed grid of kRedBlocks x 256 threads with a
// fixed-shape tree, so the same inputs give the same bits on every run; the PCG
// scalars (alpha, beta) are read from device memory, never round-tripped through
// the host.  These kernels are HBM-bound streaming passes.
#include <cuda_runtime.h>

#include <algorithm>
#include <type_traits>

#include "tg_internal.h"

namespace tg {

namespace {
constexpr int kThreads = 256;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// Deterministic block sum (fixed tree), result valid in thread 0.
__device__ __forceinline__ double block_sum256(double v) {
  __shared__ double red[kThreads / 32];
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) red[wid] = v;
  __syncthreads();
  double s = 0.0;
  if (wid == 0) {
    s = lane < kThreads / 32 ? red[lane] : 0.0;
    s = warp_sum(s);
  }
  __syncthreads();
  return s;
}

__device__ __forceinline__ double block_max256(double v) {
  __shared__ double red[kThreads / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) red[wid] = v;
  __syncthreads();
  double s = 0.0;
  if (wid == 0) {
    s = lane < kThreads / 32 ? red[lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s = fmax(s, __shfl_down_sync(0xffffffffu, s, o));
  }
  __syncthreads();
  return s;
}

// FP32 vectors are summed in FP32 along each thread's grid-stride run (a few
// dozen terms) and in FP64 across threads and blocks: on GB300 an FP64 multiply
// per element would make these streaming kernels FP64-pipe-bound.
template <class T>
__global__ void k_dot(const T* __restrict__ a, const T* __restrict__ b, int64_t n,
                      double* __restrict__ part) {
  T t = T(0);
  for (int64_t i = blockIdx.x * int64_t(kThreads) + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * kThreads)
    t += a[i] * b[i];
  const double s = block_sum256(double(t));
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// One block: out = sum of n partials, fixed order.
__global__ void k_sum_partials(const double* __restrict__ part, int n, double* __restrict__ out) {
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += kThreads) s += part[i];
  s = block_sum256(s);
  if (threadIdx.x == 0) *out = s;
}

__global__ void k_max_partials(const double* __restrict__ part, int n, double* __restrict__ out) {
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += kThreads) s = fmax(s, part[i]);
  s = block_max256(s);
  if (threadIdx.x == 0) *out = s;
}

// x += alpha p; r -= alpha Ap with alpha = rz / pAp; partial r.r (FP64 sums).
// The FP64 PCG's update; the FP32 inner PCG runs it as two kernels below.
template <class T>
__global__ void k_cg_update_xr(T* __restrict__ x, T* __restrict__ r, const T* __restrict__ p,
                               const T* __restrict__ ap, const double* __restrict__ rz,
                               const double* __restrict__ pap, int64_t n,
                               double* __restrict__ part) {
  // A non-positive or non-finite pAp is a breakdown the host reports; leave the
  // iterate untouched so the last good x survives.
  const double pp = *pap;
  const T a = T((pp > 0.0 && isfinite(pp)) ? *rz / pp : 0.0);
  T t = T(0);
  for (int64_t i = blockIdx.x * int64_t(kThreads) + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * kThreads) {
    x[i] += a * p[i];
    const T ri = r[i] - a * ap[i];
    r[i] = ri;
    t += ri * ri;
  }
  const double s = block_sum256(double(t));
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// The FP32 inner PCG's update in two kernels (alpha as k_cg_update_xr forms it,
// 16-byte vector accesses): r -= alpha Ap with partial r.r, and x += alpha p,
// which the solver runs later, beside the next V-cycle's coarse levels
// (nothing in the loop reads x).
__device__ __forceinline__ float cg_alpha_f(const double* rz, const double* pap) {
  const double pp = *pap;
  return float((pp > 0.0 && isfinite(pp)) ? *rz / pp : 0.0);
}
// With x0 set, also x0 = omega invdiag .* r (the next V-cycle's first smoothing
// sweep from zero, as k_jacobi_first computes it).
__global__ void k_cg_update_r_f(float* __restrict__ r, const float* __restrict__ ap,
                                const double* __restrict__ rz, const double* __restrict__ pap,
                                int64_t n, double* __restrict__ part,
                                const float* __restrict__ invdiag, float omega,
                                float* __restrict__ x0) {
  const float af = cg_alpha_f(rz, pap);
  const int64_t n4 = n >> 2;
  float4* r4 = reinterpret_cast<float4*>(r);
  const float4* a4 = reinterpret_cast<const float4*>(ap);
  const float4* d4 = reinterpret_cast<const float4*>(invdiag);
  float4* x4 = reinterpret_cast<float4*>(x0);
  float tf = 0.0f;
  for (int64_t i = blockIdx.x * int64_t(kThreads) + threadIdx.x; i < n4;
       i += int64_t(gridDim.x) * kThreads) {
    float4 rv = r4[i];
    const float4 qv = a4[i];
    rv.x -= af * qv.x; rv.y -= af * qv.y; rv.z -= af * qv.z; rv.w -= af * qv.w;
    r4[i] = rv;
    tf += rv.x * rv.x + rv.y * rv.y + rv.z * rv.z + rv.w * rv.w;
    if (x0 != nullptr) {
      const float4 dv = d4[i];
      x4[i] = make_float4(omega * dv.x * rv.x, omega * dv.y * rv.y, omega * dv.z * rv.z,
                          omega * dv.w * rv.w);
    }
  }
  float t = tf;
  for (int64_t i = (n4 << 2) + blockIdx.x * int64_t(kThreads) + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * kThreads) {
    const float ri = r[i] - af * ap[i];
    r[i] = ri;
    t += ri * ri;
    if (x0 != nullptr) x0[i] = omega * invdiag[i] * ri;
  }
  const double s = block_sum256(double(t));
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}
__global__ void k_cg_update_x_f(float* __restrict__ x, const float* __restrict__ p,
                                const double* __restrict__ rz, const double* __restrict__ pap,
                                int64_t n) {
  const float af = cg_alpha_f(rz, pap);
  const int64_t n4 = n >> 2;
  float4* x4 = reinterpret_cast<float4*>(x);
  const float4* p4 = reinterpret_cast<const float4*>(p);
  for (int64_t i = blockIdx.x * int64_t(kThreads) + threadIdx.x; i < n4;
       i += int64_t(gridDim.x) * kThreads) {
    float4 xv = x4[i];
    const float4 pv = p4[i];
    xv.x += af * pv.x; xv.y += af * pv.y; xv.z += af * pv.z; xv.w += af * pv.w;
    x4[i] = xv;
  }
  for (int64_t i = (n4 << 2) + blockIdx.x * int64_t(kThreads) + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * kThreads)
    x[i] += af * p[i];
}

// z = invdiag .* r (Jacobi preconditioner); partial r.z.
__global__ void k_scale_mask(double* __restrict__ z, const double* __restrict__ r,
                             const double* __restrict__ invdiag, int64_t n,
                             double* __restrict__ part) {
  double s = 0.0;
  for (int64_t i = blockIdx.x * int64_t(kThreads) + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * kThreads) {
    const double zi = invdiag[i] * r[i];
    z[i] = zi;
    s += r[i] * zi;
  }
  s = block_sum256(s);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// p = z + beta p, beta = rz_new / rz_old.
template <class T>
__global__ void k_cg_update_p(T* __restrict__ p, const T* __restrict__ z,
                              const double* __restrict__ rz_new, const double* __restrict__ rz_old,
                              int64_t n) {
  const T beta = T(*rz_new / *rz_old);
  int64_t i0 = 0;
  if (std::is_same<T, float>::value) {
    const int64_t n4 = n >> 2;
    float4* p4 = reinterpret_cast<float4*>(p);
    const float4* z4 = reinterpret_cast<const float4*>(z);
    const float b = float(beta);
    for (int64_t i = blockIdx.x * int64_t(kThreads) + threadIdx.x; i < n4;
         i += int64_t(gridDim.x) * kThreads) {
      float4 pv = p4[i];
      const float4 zv = z4[i];
      pv.x = zv.x + b * pv.x; pv.y = zv.y + b * pv.y; pv.z = zv.z + b * pv.z; pv.w = zv.w + b * pv.w;
      p4[i] = pv;
    }
    i0 = n4 << 2;
  }
  for (int64_t i = i0 + blockIdx.x * int64_t(kThreads) + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * kThreads)
    p[i] = z[i] + beta * p[i];
}

__global__ void k_scale_d2f(float* __restrict__ d, const double* __restrict__ s,
                            const double* __restrict__ nrm2, int64_t n) {
  const double inv = *nrm2 > 0.0 ? 1.0 / sqrt(*nrm2) : 0.0;
  for (int64_t i = blockIdx.x * int64_t(kThreads) + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * kThreads)
    d[i] = float(s[i] * inv);
}

// y += sqrt(*nrm2) * x (undo the scaling while accumulating in double).
__global__ void k_axpy_scaled_f2d(double* __restrict__ y, const float* __restrict__ x,
                                  const double* __restrict__ nrm2, int64_t n) {
  const double sc = sqrt(*nrm2);
  for (int64_t i = blockIdx.x * int64_t(kThreads) + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * kThreads)
    y[i] += sc * double(x[i]);
}

template <class T>
__global__ void k_fill(T* __restrict__ a, T v, int64_t n) {
  for (int64_t i = blockIdx.x * int64_t(kThreads) + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * kThreads)
    a[i] = v;
}

__global__ void k_copy_d2f(float* __restrict__ d, const double* __restrict__ s, int64_t n) {
  for (int64_t i = blockIdx.x * int64_t(kThreads) + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * kThreads)
    d[i] = float(s[i]);
}

__global__ void k_axpy_f2d(double* __restrict__ y, const float* __restrict__ x, int64_t n) {
  for (int64_t i = blockIdx.x * int64_t(kThreads) + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * kThreads)
    y[i] += double(x[i]);
}

__global__ void k_sub_mask(double* __restrict__ r, const double* __restrict__ b,
                           const double* __restrict__ ax, const uint8_t* __restrict__ kept,
                           int64_t n) {
  for (int64_t i = blockIdx.x * int64_t(kThreads) + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * kThreads)
    r[i] = kept[i] ? b[i] - ax[i] : 0.0;
}

// u = kept ? x : alt (x is also allowed to be null -> 0 on kept DOFs).
__global__ void k_mask_select(double* __restrict__ u, const double* __restrict__ x,
                              const double* __restrict__ alt, const uint8_t* __restrict__ kept,
                              int64_t n) {
  for (int64_t i = blockIdx.x * int64_t(kThreads) + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * kThreads)
    u[i] = kept[i] ? (x ? x[i] : 0.0) : (alt ? alt[i] : 0.0);
}

__global__ void k_absdiff_max(const double* __restrict__ a, const double* __restrict__ b,
                              int64_t n, double* __restrict__ part) {
  double s = 0.0;
  for (int64_t i = blockIdx.x * int64_t(kThreads) + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * kThreads)
    s = fmax(s, fabs(a[i] - b[i]));
  s = block_max256(s);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// FMA throughput probe: 8 independent register-resident FMA chains per thread.
template <class T>
__global__ void k_fma_probe(T* __restrict__ out, int iters, T b, T c) {
  T a0 = T(threadIdx.x), a1 = a0 + T(1), a2 = a0 + T(2), a3 = a0 + T(3);
  T a4 = a0 + T(4), a5 = a0 + T(5), a6 = a0 + T(6), a7 = a0 + T(7);
  for (int i = 0; i < iters; ++i) {
    a0 = fma(a0, b, c); a1 = fma(a1, b, c); a2 = fma(a2, b, c); a3 = fma(a3, b, c);
    a4 = fma(a4, b, c); a5 = fma(a5, b, c); a6 = fma(a6, b, c); a7 = fma(a7, b, c);
  }
  const T s = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
  if (s == T(-1.2345)) out[blockIdx.x] = s;  // keeps the chains live
}

int stream_blocks(int64_t n) {
  const int64_t b = (n + kThreads - 1) / kThreads;
  return int(b < kRedBlocks ? (b > 0 ? b : 1) : kRedBlocks);
}
}  // namespace

double fma_probe_tflops(bool fp64) {
  const int blocks = 152 * 8, threads = 256;
  const int iters = fp64 ? 4096 : 262144;
  void* out = nullptr;
  TG_CUDA(cudaMalloc(&out, blocks * sizeof(double)));
  cudaEvent_t a, b;
  TG_CUDA(cudaEventCreate(&a));
  TG_CUDA(cudaEventCreate(&b));
  double best = 0.0;
  for (int rep = 0; rep < 3; ++rep) {
    TG_CUDA(cudaEventRecord(a));
    if (fp64)
      k_fma_probe<double><<<blocks, threads>>>(static_cast<double*>(out), iters, 0.999999, 1e-7);
    else
      k_fma_probe<float><<<blocks, threads>>>(static_cast<float*>(out), iters, 0.999999f, 1e-7f);
    TG_LAUNCH_CHECK();
    TG_CUDA(cudaEventRecord(b));
    TG_CUDA(cudaEventSynchronize(b));
    float ms = 0.0f;
    TG_CUDA(cudaEventElapsedTime(&ms, a, b));
    const double flops = 2.0 * 8.0 * double(iters) * blocks * threads;
    best = std::max(best, flops / (double(ms) * 1e-3) / 1e12);
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(out);
  return best;
}

void launch_dot(const double* a, const double* b, int64_t n, double* part, double* out,
                cudaStream_t s) {
  k_dot<double><<<kRedBlocks, kThreads, 0, s>>>(a, b, n, part);
  TG_LAUNCH_CHECK();
  k_sum_partials<<<1, kThreads, 0, s>>>(part, kRedBlocks, out);
  TG_LAUNCH_CHECK();
}

void launch_dot_f(const float* a, const float* b, int64_t n, double* part, double* out,
                  cudaStream_t s) {
  k_dot<float><<<kRedBlocks, kThreads, 0, s>>>(a, b, n, part);
  TG_LAUNCH_CHECK();
  k_sum_partials<<<1, kThreads, 0, s>>>(part, kRedBlocks, out);
  TG_LAUNCH_CHECK();
}

void launch_dot_partials_f(const float* a, const float* b, int64_t n, double* part,
                           cudaStream_t s) {
  k_dot<float><<<kRedBlocks, kThreads, 0, s>>>(a, b, n, part);
  TG_LAUNCH_CHECK();
}

void launch_sum_partials(const double* part, int n, double* out, cudaStream_t s) {
  k_sum_partials<<<1, kThreads, 0, s>>>(part, n, out);
  TG_LAUNCH_CHECK();
}

template <class T>
void launch_cg_update_xr(T* x, T* r, const T* p, const T* ap, const double* rz,
                         const double* pap, int64_t n, double* rr_part, cudaStream_t s) {
  k_cg_update_xr<T><<<kRedBlocks, kThreads, 0, s>>>(x, r, p, ap, rz, pap, n, rr_part);
  TG_LAUNCH_CHECK();
}
template void launch_cg_update_xr<double>(double*, double*, const double*, const double*,
                                          const double*, const double*, int64_t, double*,
                                          cudaStream_t);

void launch_cg_update_r_f(float* r, const float* ap, const double* rz, const double* pap,
                          int64_t n, double* rr_part, cudaStream_t s, const float* invdiag,
                          float omega, float* x0) {
  k_cg_update_r_f<<<kRedBlocks, kThreads, 0, s>>>(r, ap, rz, pap, n, rr_part, invdiag, omega,
                                                  x0);
  TG_LAUNCH_CHECK();
}
void launch_cg_update_x_f(float* x, const float* p, const double* rz, const double* pap,
                          int64_t n, cudaStream_t s) {
  k_cg_update_x_f<<<kRedBlocks, kThreads, 0, s>>>(x, p, rz, pap, n);
  TG_LAUNCH_CHECK();
}

void launch_scale_mask(double* z, const double* r, const double* invdiag, int64_t n,
                       double* rz_part, cudaStream_t s) {
  k_scale_mask<<<kRedBlocks, kThreads, 0, s>>>(z, r, invdiag, n, rz_part);
  TG_LAUNCH_CHECK();
}

template <class T>
void launch_cg_update_p(T* p, const T* z, const double* rz_new, const double* rz_old, int64_t n,
                        cudaStream_t s) {
  k_cg_update_p<T><<<kRedBlocks, kThreads, 0, s>>>(p, z, rz_new, rz_old, n);
  TG_LAUNCH_CHECK();
}
template void launch_cg_update_p<double>(double*, const double*, const double*, const double*,
                                         int64_t, cudaStream_t);
template void launch_cg_update_p<float>(float*, const float*, const double*, const double*,
                                        int64_t, cudaStream_t);

void launch_scale_d2f(float* dst, const double* src, const double* nrm2, int64_t n,
                      cudaStream_t s) {
  k_scale_d2f<<<stream_blocks(n), kThreads, 0, s>>>(dst, src, nrm2, n);
  TG_LAUNCH_CHECK();
}

void launch_axpy_scaled_f2d(double* y, const float* x, const double* nrm2, int64_t n,
                            cudaStream_t s) {
  k_axpy_scaled_f2d<<<stream_blocks(n), kThreads, 0, s>>>(y, x, nrm2, n);
  TG_LAUNCH_CHECK();
}

template <class T>
void launch_fill(T* a, T v, int64_t n, cudaStream_t s) {
  k_fill<T><<<stream_blocks(n), kThreads, 0, s>>>(a, v, n);
  TG_LAUNCH_CHECK();
}
template void launch_fill<double>(double*, double, int64_t, cudaStream_t);
template void launch_fill<float>(float*, float, int64_t, cudaStream_t);
template void launch_fill<uint8_t>(uint8_t*, uint8_t, int64_t, cudaStream_t);

void launch_copy_d2f(float* dst, const double* src, int64_t n, cudaStream_t s) {
  k_copy_d2f<<<stream_blocks(n), kThreads, 0, s>>>(dst, src, n);
  TG_LAUNCH_CHECK();
}

void launch_axpy_f2d(double* y, const float* x, int64_t n, cudaStream_t s) {
  k_axpy_f2d<<<stream_blocks(n), kThreads, 0, s>>>(y, x, n);
  TG_LAUNCH_CHECK();
}

void launch_sub_mask(double* r, const double* b, const double* ax, const uint8_t* kept, int64_t n,
                     cudaStream_t s) {
  k_sub_mask<<<stream_blocks(n), kThreads, 0, s>>>(r, b, ax, kept, n);
  TG_LAUNCH_CHECK();
}

void launch_mask_select(double* u, const double* x, const double* alt, const uint8_t* kept,
                        int64_t n, cudaStream_t s) {
  k_mask_select<<<stream_blocks(n), kThreads, 0, s>>>(u, x, alt, kept, n);
  TG_LAUNCH_CHECK();
}

void launch_absdiff_max(const double* a, const double* b, int64_t n, double* part, double* out,
                        cudaStream_t s) {
  k_absdiff_max<<<kRedBlocks, kThreads, 0, s>>>(a, b, n, part);
  TG_LAUNCH_CHECK();
  k_max_partials<<<1, kThreads, 0, s>>>(part, kRedBlocks, out);
  TG_LAUNCH_CHECK();
}

}  // namespace tg
