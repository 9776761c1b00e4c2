// k_operator.cu -- the matrix-free hex8 operator on the voxel grid.
//
// Reference counterpart: mf_apply_full / apply_one_element / axpy24
// (core/src/fea/matfree.cpp:535-553, :110-123, :75-96) and the reduced-system
// matvec apply_kgg_raw (matfree.cpp:595-608).  The reference multiplies every
// element's 24 DOFs by the dense 24x24 Ke (576 mul+add per element).  Here the
// same operator is evaluated in the Walsh-modal basis of the trilinear element:
//
//   u(xi) = sum_S m[S] prod_{i in S} xi_i,   S subset of {x,y,z}   (8 modes)
//
// The gradient coefficient of monomial T in du_j/dxi_i is m_j[T u {i}], and the
// monomials are orthogonal on the cube, so the 2x2x2-Gauss strain energy splits
// into independent blocks per T with weights 8/3^|T|.  K u is the gradient of
// that energy: a forward Walsh transform (24 add/sub per component), about 50
// flops of isotropic "stress" per element, and the inverse transform.  About 200
// floating-point operations replace 576 FMAs -- it matters because GB300 runs
// FP64 at roughly 1/64 of its FP32 rate.  The result equals Ke u to rounding
// (checked against the oracle's dense Ke in the tests).
//
// Scheduling: x-pencils marching in z (see k_fine_op below): element outputs are
// combined along x by warp shuffles, along y through shared memory and along z
// in registers, so each node is finished exactly once without atomics and the
// per-node summation order is fixed -- the apply is deterministic run to run.
#include <cuda_runtime.h>

#include <algorithm>
#include <type_traits>

#include "tg_df.h"
#include "tg_internal.h"

namespace tg {

ModalConsts ModalConsts::make(double nu, double h) {
  ModalConsts c;
  const double lam = nu / ((1.0 + nu) * (1.0 - 2.0 * nu));
  const double mu = 1.0 / (2.0 * (1.0 + nu));
  double s = h / 16.0;
  for (int k = 0; k < 3; ++k) {
    c.L[k] = lam * s;
    c.M[k] = mu * s;
    s /= 3.0;
  }
  c.kdiag = 0.0;  // filled by the caller from the unit-modulus Ke (all 24 equal)
  return c;
}

template <class T>
struct ModalT {
  T L0, L1, M0, M1, M02, M12, LM2;  // per unit modulus; M02 = 2*M0, LM2 = L2 + 4*M2
};

// Storage (T) to compute (C) and back: the identity, except that a double is
// carried as a double-float (tg_df.h) by the residual-only instantiation.
template <class C>
__host__ __device__ __forceinline__ C cvt(double v) {
  return C(v);
}
template <>
__host__ __device__ __forceinline__ df cvt<df>(double v) {
  return df_from(v);
}
template <class C, class T>
__device__ __forceinline__ C load_c(T v) {
  return cvt<C>(v);
}
template <>
__device__ __forceinline__ float load_c<float, float>(float v) {
  return v;
}
__device__ __forceinline__ double store_t(double v) { return v; }
__device__ __forceinline__ float store_t(float v) { return v; }
__device__ __forceinline__ double store_t(df v) { return df_to_double(v); }
__device__ __forceinline__ bool nonzero(float v) { return v != 0.0f; }
__device__ __forceinline__ bool nonzero(double v) { return v != 0.0; }
__device__ __forceinline__ bool nonzero(df v) { return df_nonzero(v); }
__device__ __forceinline__ float shfl_up(float v, int d) { return __shfl_up_sync(0xffffffffu, v, d); }
__device__ __forceinline__ double shfl_up(double v, int d) { return __shfl_up_sync(0xffffffffu, v, d); }
__device__ __forceinline__ float shfl_down(float v, int d) {
  return __shfl_down_sync(0xffffffffu, v, d);
}
__device__ __forceinline__ double shfl_down(double v, int d) {
  return __shfl_down_sync(0xffffffffu, v, d);
}
template <class C>
__host__ __device__ __forceinline__ C czero() {
  return cvt<C>(0.0);
}

template <class T>
ModalT<T> to_modal(const ModalConsts& c) {
  ModalT<T> m;
  m.L0 = cvt<T>(c.L[0]);
  m.L1 = cvt<T>(c.L[1]);
  m.M0 = cvt<T>(c.M[0]);
  m.M1 = cvt<T>(c.M[1]);
  m.M02 = cvt<T>(2.0 * c.M[0]);
  m.M12 = cvt<T>(2.0 * c.M[1]);
  m.LM2 = cvt<T>(c.L[2] + 4.0 * c.M[2]);
  return m;
}

// a * b + c, spelled out so the modal arithmetic below maps to fused multiply-adds.
__device__ __forceinline__ float mad(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double mad(double a, double b, double c) { return fma(a, b, c); }

// Forward Walsh transform of one component: v[idx], idx = sx | sy<<1 | sz<<2
// with s = 1 on the + side, becomes the unnormalised mode coefficients
// 8*m[mask], mask bit i set when axis i is in the monomial.
template <class T>
__device__ __forceinline__ void walsh_fwd(T (&v)[8]) {
#pragma unroll
  for (int b = 1; b < 8; b <<= 1) {
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      if (i & b) continue;
      const T lo = v[i], hi = v[i | b];
      v[i] = hi + lo;
      v[i | b] = hi - lo;
    }
  }
}

// Inverse (unnormalised) transform: corner values from mode coefficients.
template <class T>
__device__ __forceinline__ void walsh_inv(T (&w)[8]) {
#pragma unroll
  for (int b = 1; b < 8; b <<= 1) {
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      if (i & b) continue;
      const T lo = w[i], hi = w[i | b];
      w[i] = lo - hi;
      w[i | b] = lo + hi;
    }
  }
}

// out = f * Ke * u for one element; u and out indexed [corner idx][comp].
template <class T>
__device__ __forceinline__ void modal_apply(const ModalT<T>& mc, T f, T (&ux)[8], T (&uy)[8],
                                            T (&uz)[8]) {
  walsh_fwd(ux);
  walsh_fwd(uy);
  walsh_fwd(uz);
  const T L0 = mc.L0 * f, L1 = mc.L1 * f, M0 = mc.M0 * f, M1 = mc.M1 * f;
  const T M02 = mc.M02 * f, M12 = mc.M12 * f, LM2 = mc.LM2 * f;
  T gx[8], gy[8], gz[8];
  // |T| = 0: the constant-gradient block.
  {
    const T Ltr = L0 * (ux[1] + uy[2] + uz[4]);
    gx[1] = mad(M02, ux[1], Ltr);
    gy[2] = mad(M02, uy[2], Ltr);
    gz[4] = mad(M02, uz[4], Ltr);
    const T txy = M0 * (uy[1] + ux[2]);
    const T txz = M0 * (uz[1] + ux[4]);
    const T tyz = M0 * (uz[2] + uy[4]);
    gy[1] = txy; gz[1] = txz;
    gx[2] = txy; gz[2] = tyz;
    gx[4] = txz; gy[4] = tyz;
  }
  // |T| = 1: gradients linear along one axis; modes 3, 5, 6 each get two terms.
  {
    const T Ltr = L1 * (uy[3] + uz[5]);  // T = {x}: rows y (mode 3), z (mode 5)
    const T t = M1 * (uz[3] + uy[5]);
    gx[3] = M1 * ux[3];
    gy[3] = mad(M12, uy[3], Ltr);
    gz[3] = t;
    gx[5] = M1 * ux[5];
    gy[5] = t;
    gz[5] = mad(M12, uz[5], Ltr);
  }
  {
    const T Ltr = L1 * (ux[3] + uz[6]);  // T = {y}: rows x (mode 3), z (mode 6)
    const T t = M1 * (uz[3] + ux[6]);
    gx[3] = gx[3] + mad(M12, ux[3], Ltr);
    gy[3] = mad(M1, uy[3], gy[3]);
    gz[3] = gz[3] + t;
    gx[6] = t;
    gy[6] = M1 * uy[6];
    gz[6] = mad(M12, uz[6], Ltr);
  }
  {
    const T Ltr = L1 * (ux[5] + uy[6]);  // T = {z}: rows x (mode 5), y (mode 6)
    const T t = M1 * (uy[5] + ux[6]);
    gx[5] = gx[5] + mad(M12, ux[5], Ltr);
    gy[5] = gy[5] + t;
    gz[5] = mad(M1, uz[5], gz[5]);
    gx[6] = gx[6] + t;
    gy[6] = gy[6] + mad(M12, uy[6], Ltr);
    gz[6] = mad(M1, uz[6], gz[6]);
  }
  // |T| = 2: the trilinear mode.
  gx[7] = LM2 * ux[7];
  gy[7] = LM2 * uy[7];
  gz[7] = LM2 * uz[7];
  gx[0] = gy[0] = gz[0] = czero<T>();
  walsh_inv(gx);
  walsh_inv(gy);
  walsh_inv(gz);
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    ux[i] = gx[i];
    uy[i] = gy[i];
    uz[i] = gz[i];
  }
}

// ---- the same element operator with the x and y components packed ----
// Blackwell's paired FP32 instructions (FADD2/FMUL2/FFMA2) operate on a float2
// as one instruction.  The Walsh transforms treat x and y identically, so they
// run on (x, y) pairs; the isotropic "stress" block mixes components and stays
// scalar.  Same operations per component as modal_apply, same rounding.
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) {
  return __ffma2_rn(b, make_float2(-1.0f, -1.0f), a);  // a - b, one rounding
}
__device__ __forceinline__ void walsh_fwd2(float2 (&v)[8]) {
#pragma unroll
  for (int b = 1; b < 8; b <<= 1) {
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      if (i & b) continue;
      const float2 lo = v[i], hi = v[i | b];
      v[i] = add2(hi, lo);
      v[i | b] = sub2(hi, lo);
    }
  }
}
__device__ __forceinline__ void walsh_inv2(float2 (&w)[8]) {
#pragma unroll
  for (int b = 1; b < 8; b <<= 1) {
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      if (i & b) continue;
      const float2 lo = w[i], hi = w[i | b];
      w[i] = sub2(lo, hi);
      w[i | b] = add2(lo, hi);
    }
  }
}
__device__ __forceinline__ void modal_apply_xy(const ModalT<float>& mc, float f, float2 (&uxy)[8],
                                               float (&uz)[8]) {
  walsh_fwd2(uxy);
  walsh_fwd(uz);
  const float L0 = mc.L0 * f, L1 = mc.L1 * f, M0 = mc.M0 * f, M1 = mc.M1 * f;
  const float M02 = mc.M02 * f, M12 = mc.M12 * f, LM2 = mc.LM2 * f;
  float2 g[8];
  float gz[8];
  {
    const float Ltr = L0 * (uxy[1].x + uxy[2].y + uz[4]);
    g[1].x = mad(M02, uxy[1].x, Ltr);
    g[2].y = mad(M02, uxy[2].y, Ltr);
    gz[4] = mad(M02, uz[4], Ltr);
    const float txy = M0 * (uxy[1].y + uxy[2].x);
    const float txz = M0 * (uz[1] + uxy[4].x);
    const float tyz = M0 * (uz[2] + uxy[4].y);
    g[1].y = txy; gz[1] = txz;
    g[2].x = txy; gz[2] = tyz;
    g[4].x = txz; g[4].y = tyz;
  }
  {
    const float Ltr = L1 * (uxy[3].y + uz[5]);
    const float t = M1 * (uz[3] + uxy[5].y);
    g[3].x = M1 * uxy[3].x;
    g[3].y = mad(M12, uxy[3].y, Ltr);
    gz[3] = t;
    g[5].x = M1 * uxy[5].x;
    g[5].y = t;
    gz[5] = mad(M12, uz[5], Ltr);
  }
  {
    const float Ltr = L1 * (uxy[3].x + uz[6]);
    const float t = M1 * (uz[3] + uxy[6].x);
    g[3].x = g[3].x + mad(M12, uxy[3].x, Ltr);
    g[3].y = mad(M1, uxy[3].y, g[3].y);
    gz[3] = gz[3] + t;
    g[6].x = t;
    g[6].y = M1 * uxy[6].y;
    gz[6] = mad(M12, uz[6], Ltr);
  }
  {
    const float Ltr = L1 * (uxy[5].x + uxy[6].y);
    const float t = M1 * (uxy[5].y + uxy[6].x);
    g[5].x = g[5].x + mad(M12, uxy[5].x, Ltr);
    g[5].y = g[5].y + t;
    gz[5] = mad(M1, uz[5], gz[5]);
    g[6].x = g[6].x + t;
    g[6].y = g[6].y + mad(M12, uxy[6].y, Ltr);
    gz[6] = mad(M1, uz[6], gz[6]);
  }
  g[7] = __fmul2_rn(make_float2(LM2, LM2), uxy[7]);
  gz[7] = LM2 * uz[7];
  g[0] = make_float2(0.0f, 0.0f);
  gz[0] = 0.0f;
  walsh_inv2(g);
  walsh_inv(gz);
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    uxy[i] = g[i];
    uz[i] = gz[i];
  }
}

struct GridDev {
  int nx, ny, nz, nnx, nny, nnz;
};

// Batched periodic applies (homogenization): system bi of the batch reads x, b,
// y at bi * sx and the cell fields (factors, kept mask, inverse diagonal) of
// cell bi / nrhs.  On the torus nodes and elements coincide (nnx == nx ...).
struct BatchDev {
  int nrhs, nzc;         // systems per cell; z-chunks per system
  int64_t sx, se, sk;    // strides: DOF vectors, element factors, per-cell DOF fields
};

__device__ __forceinline__ int wrap_index(int a, int n) {
  a %= n;
  return a < 0 ? a + n : a;
}

__device__ __forceinline__ double block_sum(double v) {
  __shared__ double red[32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[wid] = v;
  __syncthreads();
  double s = 0.0;
  if (wid == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    s = lane < nw ? red[lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  }
  return s;  // valid in thread 0
}

// Pencil geometry.  A CTA is PY warps.  Lane l of warp w evaluates the elements
// (ex, ey, ez) with ex = 31*bx - 1 + l and ey = (PY-1)*by - 1 + w for KZ+1
// consecutive element layers, marching upward in z.  Contributions are combined
//   along x by a warp shuffle (an element's +x corners belong to the next lane),
//   along y through shared memory (a warp's +y corners belong to the next warp),
//   along z in registers (a layer's +z corners wait for the next step),
// so lane l >= 1 of warp w >= 1 finishes node (ex, ey, ez) once element layers
// ez-1 and ez are in.  Lane 0, warp 0 and the first element layer are the halo:
// recomputed, never written.  One __syncthreads per element layer, no atomics,
// and a fixed summation order per node (x, then y, then z), so the result is
// deterministic run to run.
template <class T>
struct Pencil;
template <>
struct Pencil<double> {
  static constexpr int PY = 8, KZ = 16, MINB = 2;
};
#ifndef TG_PENCIL_F32_PY
#define TG_PENCIL_F32_PY 8
#endif
#ifndef TG_PENCIL_F32_KZ
#define TG_PENCIL_F32_KZ 16
#endif
#ifndef TG_PENCIL_F32_MINB
#define TG_PENCIL_F32_MINB 3
#endif
template <>
struct Pencil<float> {
  static constexpr int PY = TG_PENCIL_F32_PY, KZ = TG_PENCIL_F32_KZ, MINB = TG_PENCIL_F32_MINB;
};
template <>
struct Pencil<df> {
  static constexpr int PY = 8, KZ = 16, MINB = 2;
};

template <class T, bool PER = false>
__device__ __forceinline__ void load_node(const GridDev& g, const T* __restrict__ x, int a, int b,
                                          int c, T (&v)[3]) {
  if (PER) {
    a = wrap_index(a, g.nnx);
    b = wrap_index(b, g.nny);
    c = wrap_index(c, g.nnz);
  }
  if (PER || (a >= 0 && a < g.nnx && b >= 0 && b < g.nny && c >= 0 && c < g.nnz)) {
    const T* p = x + 3 * ((int64_t(c) * g.nny + b) * g.nnx + a);
    v[0] = p[0];
    v[1] = p[1];
    v[2] = p[2];
  } else {
    v[0] = v[1] = v[2] = T(0);
  }
}

// Raw loads of layer c for the lane's own column: nodes (ex, ey, c), (ex, ey+1, c)
// and, for lane 31, (ex+1, ey, c), (ex+1, ey+1, c).  Issued one step ahead so
// their latency overlaps the current layer's arithmetic.
template <class T, bool PER = false>
__device__ __forceinline__ void load_raw(const GridDev& g, const T* __restrict__ x, int ex, int ey,
                                         int c, int lane, T (&r)[2][2][3]) {
  load_node<T, PER>(g, x, ex, ey, c, r[0][0]);
  load_node<T, PER>(g, x, ex, ey + 1, c, r[1][0]);
  if (lane == 31) {
    load_node<T, PER>(g, x, ex + 1, ey, c, r[0][1]);
    load_node<T, PER>(g, x, ex + 1, ey + 1, c, r[1][1]);
  }
}

// The same loads for the non-periodic grid with the column's x/y validity
// (m[yb][xb]) and base offset hoisted out of the z march: layer c adds
// 3*c*nnx*nny to the offset and tests only its own z range.
template <class T, class C>
__device__ __forceinline__ void load_raw_np(const T* __restrict__ x, int64_t o, int snx, bool vc,
                                            const bool (&m)[2][2], int lane, C (&r)[2][2][3]) {
#pragma unroll
  for (int yb = 0; yb < 2; ++yb)
#pragma unroll
    for (int xb = 0; xb < 2; ++xb) {
      if (xb == 1 && lane != 31) continue;
      const bool ok = vc && m[yb][xb];
      const T* p = x + (o + yb * snx + 3 * xb);
#pragma unroll
      for (int k = 0; k < 3; ++k) r[yb][xb][k] = ok ? load_c<C>(p[k]) : czero<C>();
    }
}

// Completes a layer: v[yb][xb][comp] for nodes (ex + xb, ey + yb); the +x nodes
// come from the next lane (lane 31 loaded its own).
template <class T>
__device__ __forceinline__ void finish_layer(int lane, const T (&r)[2][2][3], T (&v)[2][2][3]) {
#pragma unroll
  for (int yb = 0; yb < 2; ++yb)
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      v[yb][0][k] = r[yb][0][k];
      const T nb = shfl_down(r[yb][0][k], 1);
      v[yb][1][k] = lane == 31 ? r[yb][1][k] : nb;
    }
}

// PER: the periodic (torus) grid of a batch of systems (BatchDev); nodes and
// elements wrap around, so every element exists and the halo lanes read the
// opposite face.  The non-periodic instantiations compile the PER branches away.
template <class T, int PY, int KZ, int MINB, int MODE, bool PER = false, class C = T>
__global__ void __launch_bounds__(32 * PY, MINB) k_fine_op(GridDev g, ModalT<C> mc,
                                                     const T* __restrict__ ef,
                                                     const uint8_t* __restrict__ kept,
                                                     const T* __restrict__ x, const T* __restrict__ b,
                                                     const T* __restrict__ invdiag, T omega,
                                                     T* __restrict__ y, double* __restrict__ dot_part,
                                                     BatchDev bd = BatchDev{}) {
  __shared__ C sy[2][PY][6][32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int ex = blockIdx.x * 31 - 1 + lane;
  const int ey = blockIdx.y * (PY - 1) - 1 + w;
  int k0 = blockIdx.z * KZ;
  if (PER) {
    const int bi = blockIdx.z / bd.nzc, cell = bi / bd.nrhs;
    k0 = (blockIdx.z - bi * bd.nzc) * KZ;
    x += bi * bd.sx;
    y += bi * bd.sx;
    if (b) b += bi * bd.sx;
    ef += cell * bd.se;
    if (kept) kept += cell * bd.sk;
    if (invdiag) invdiag += cell * bd.sk;
  }
  const bool own_xy = lane >= 1 && w >= 1 && ex < g.nnx && ey < g.nny;
  const bool exy_ok = PER || (ex >= 0 && ex < g.nx && ey >= 0 && ey < g.ny);
  const int64_t exy = PER ? int64_t(wrap_index(ey, g.ny)) * g.nx + wrap_index(ex, g.nx)
                          : int64_t(ey) * g.nx + ex;
  // Non-periodic: hoisted column validity and running offsets (nodes: o_x,
  // outputs: o_y, element factors: o_e).
  const int64_t plane3 = 3 * int64_t(g.nnx) * g.nny, eplane = int64_t(g.nx) * g.ny;
  const int snx = 3 * g.nnx;
  const bool vx0 = ex >= 0 && ex < g.nnx, vx1 = ex + 1 < g.nnx;
  const bool vy0 = ey >= 0 && ey < g.nny, vy1 = ey + 1 < g.nny;
  const bool msk[2][2] = {{vx0 && vy0, vx1 && vy0}, {vx0 && vy1, vx1 && vy1}};
  const int64_t oxy = 3 * (int64_t(ey) * g.nnx + ex);
  C cur[2][2][3], nxt[2][2][3], raw[2][2][3];
  if constexpr (PER) {
    load_raw<T, PER>(g, x, ex, ey, k0 - 1, lane, raw);
  } else {
    load_raw_np(x, oxy + (k0 - 1) * plane3, snx, k0 - 1 >= 0 && k0 - 1 < g.nnz, msk, lane, raw);
  }
  finish_layer(lane, raw, cur);
  if constexpr (PER)
    load_raw<T, PER>(g, x, ex, ey, k0, lane, raw);
  else
    load_raw_np(x, oxy + k0 * plane3, snx, k0 < g.nnz, msk, lane, raw);
  C pend[3] = {czero<C>(), czero<C>(), czero<C>()};
  C dsum = czero<C>();  // this thread's share of x.y: a few dozen nodes, then FP64 across the CTA
#pragma unroll 1
  for (int s = 0; s <= KZ; ++s) {
    const int ez = k0 - 1 + s;
    finish_layer(lane, raw, nxt);
    if (s < KZ) {
      if constexpr (PER)
        load_raw<T, PER>(g, x, ex, ey, ez + 2, lane, raw);
      else
        load_raw_np(x, oxy + (ez + 2) * plane3, snx, ez + 2 < g.nnz, msk, lane, raw);
    }
    C ux[8], uy[8], uz[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      const int xb = c & 1, yb = (c >> 1) & 1, zb = c >> 2;
      ux[c] = zb ? nxt[yb][xb][0] : cur[yb][xb][0];
      uy[c] = zb ? nxt[yb][xb][1] : cur[yb][xb][1];
      uz[c] = zb ? nxt[yb][xb][2] : cur[yb][xb][2];
    }
    C f;
    if constexpr (PER)
      f = load_c<C>(ef[int64_t(wrap_index(ez, g.nz)) * g.ny * g.nx + exy]);
    else
      f = (exy_ok && ez >= 0 && ez < g.nz) ? load_c<C>(ef[ez * eplane + exy]) : czero<C>();
    if (nonzero(f)) {
      modal_apply(mc, f, ux, uy, uz);
    } else {
#pragma unroll
      for (int c = 0; c < 8; ++c) ux[c] = uy[c] = uz[c] = czero<C>();
    }
    // x: add the previous lane's +x corners to this lane's -x corners.
    C L[2][2][3];  // [yb][zb][comp] at node x = ex
#pragma unroll
    for (int yb = 0; yb < 2; ++yb)
#pragma unroll
      for (int zb = 0; zb < 2; ++zb) {
        const int c0 = (yb << 1) | (zb << 2);
        L[yb][zb][0] = ux[c0] + shfl_up(ux[c0 | 1], 1);
        L[yb][zb][1] = uy[c0] + shfl_up(uy[c0 | 1], 1);
        L[yb][zb][2] = uz[c0] + shfl_up(uz[c0 | 1], 1);
      }
    // y: hand the +y corners to the next warp through shared memory.
    const int buf = s & 1;
#pragma unroll
    for (int zb = 0; zb < 2; ++zb)
#pragma unroll
      for (int k = 0; k < 3; ++k) sy[buf][w][zb * 3 + k][lane] = L[1][zb][k];
    __syncthreads();
    C N[2][3];
#pragma unroll
    for (int zb = 0; zb < 2; ++zb)
#pragma unroll
      for (int k = 0; k < 3; ++k)
        N[zb][k] = L[0][zb][k] + (w >= 1 ? sy[buf][w - 1][zb * 3 + k][lane] : czero<C>());
    // z: node layer ez is complete (element layers ez-1 and ez).
    if (s >= 1 && own_xy && ez < g.nnz) {
      const int64_t d0 = oxy + ez * plane3;
      C node_dot = czero<C>();  // x.y over the node's 3 DOFs, accumulated in FP64 below
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const int64_t d = d0 + k;
        const bool kk = kept == nullptr || kept[d] != 0;
        const C ax = pend[k] + N[0][k];
        T out;
        if constexpr (MODE == kApply) {
          out = kk ? store_t(ax) : T(0);
          node_dot = node_dot + cur[0][0][k] * load_c<C>(out);
        } else if constexpr (MODE == kResidual) {
          // Residual in the storage type: a double-float sum is rounded to FP64 once.
          out = kk ? T(b[d] - store_t(ax)) : T(0);
        } else {
          out = kk ? T(store_t(cur[0][0][k]) + omega * invdiag[d] * (b[d] - store_t(ax))) : T(0);
        }
        y[d] = out;
      }
      if constexpr (MODE == kApply) dsum = dsum + node_dot;
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) pend[k] = N[1][k];
#pragma unroll
    for (int yb = 0; yb < 2; ++yb)
#pragma unroll
      for (int xb = 0; xb < 2; ++xb)
#pragma unroll
        for (int k = 0; k < 3; ++k) cur[yb][xb][k] = nxt[yb][xb][k];
  }
  if (MODE == kApply && dot_part != nullptr) {
    const double sum = block_sum(double(store_t(dsum)));
    if (threadIdx.x == 0)
      dot_part[(int64_t(blockIdx.z) * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x] = sum;
  }
}

// ---------------------------------------------------------------------------
// Column-blocked FP32 operator (the mixed form's fine level).
//
// The pencil kernel above spends most of its issue slots on moving node values
// between lanes and warps and recomputes 37% of its element slots as halo.  This
// schedule keeps more of the combine in registers:
//   * lanes run along x: lane l evaluates the element column ex = x0 - 1 + l and
//     finishes node column ex (lanes 1..30; lane 0 and lane 31 are halo);
//   * each thread marches a column of Y element rows in y: the y-combine of two
//     consecutive element rows is a register add inside the thread, and an
//     element's inputs share the node row with the element below it;
//   * W warps stack in y; the node row between two warps is finished by the
//     lower warp with the upper warp's contribution handed over through shared
//     memory (one __syncthreads per element layer), so a CTA recomputes one
//     element row of halo in y, not one per warp;
//   * the CTA marches KZ element layers in z (KZ chosen per grid so the chunks
//     divide the node layers evenly), completing node layers in registers.
// Per node the summation order is fixed (y inside the thread, then x across
// lanes, then the warp hand-over, then z), so the apply is deterministic.
// Node values of layer ez+2 are loaded while layer ez is evaluated.
template <int Y, int W>
struct ColShape {
  static constexpr int kRows = W * Y - 1;  // node rows a CTA finishes
  static constexpr int kMinB = 12 / W > 0 ? 12 / W : 1;  // ~12 resident warps per SM
};

template <int Y, int W, int MODE, bool PK>
__global__ void __launch_bounds__(32 * W, (ColShape<Y, W>::kMinB))
    k_fine_op_col(GridDev g, ModalT<float> mc, int KZ, const float* __restrict__ ef,
                  const uint8_t* __restrict__ kept, const uint8_t* __restrict__ kn,
                  const float* __restrict__ x, const float* __restrict__ b,
                  const float* __restrict__ invdiag, float omega, float* __restrict__ y,
                  double* __restrict__ dot_part) {
  __shared__ float xs[2][W][6][32];
  // Smoothing with dot_part set: partial b . y as well (the PCG's r . z).
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int ex = blockIdx.x * 30 - 1 + lane;
  const int ey0 = blockIdx.y * ColShape<Y, W>::kRows - 1 + w * Y;  // element rows ey0 .. ey0+Y-1
  const int z0 = blockIdx.z * KZ;
  const int64_t plane = int64_t(g.nnx) * g.nny, eplane = int64_t(g.nx) * g.ny;
  const bool vx = ex >= 0 && ex < g.nnx;
  const bool own_x = lane >= 1 && lane <= 30 && ex < g.nnx;
  bool rv[Y + 1];
#pragma unroll
  for (int i = 0; i <= Y; ++i) rv[i] = vx && ey0 + i >= 0 && ey0 + i < g.nny;
  bool ev[Y];
#pragma unroll
  for (int j = 0; j < Y; ++j) ev[j] = ex >= 0 && ex < g.nx && ey0 + j >= 0 && ey0 + j < g.ny;
  // Node rows i = 1..Y of the column are this thread's (row Y only below the
  // top warp); row 0 belongs to the warp below.
  bool ro[Y + 1];
#pragma unroll
  for (int i = 0; i <= Y; ++i) ro[i] = own_x && i >= 1 && (i < Y || w < W - 1) && ey0 + i < g.nny;
  const int64_t col = int64_t(ey0) * g.nnx + ex;  // node (ex, ey0) in a layer
  const int64_t ecol = int64_t(ey0) * g.nx + ex;   // element (ex, ey0) in a layer

  auto load_layer = [&](int c, float (&r)[Y + 1][3]) {
    const bool vc = c >= 0 && c < g.nnz;
    const float* p = x + 3 * (int64_t(c) * plane + col);
#pragma unroll
    for (int i = 0; i <= Y; ++i)
#pragma unroll
      for (int k = 0; k < 3; ++k) r[i][k] = (vc && rv[i]) ? p[3 * i * g.nnx + k] : 0.0f;
  };
  // Element factors of layer c (0 outside the grid).
  auto load_f = [&](int c, float (&f)[Y]) {
    const bool vc = c >= 0 && c < g.nz;
#pragma unroll
    for (int j = 0; j < Y; ++j)
      f[j] = (vc && ev[j]) ? ef[int64_t(c) * eplane + ecol + int64_t(j) * g.nx] : 0.0f;
  };
  // Kept bits of the owned node rows of layer c (bit k: DOF k kept; all kept
  // without a mask).
  auto load_kb = [&](int c, unsigned (&kb)[Y + 1]) {
    const bool vc = c >= 0 && c < g.nnz;
#pragma unroll
    for (int i = 1; i <= Y; ++i)
      kb[i] = kn == nullptr ? 7u
                            : ((vc && ro[i]) ? unsigned(kn[int64_t(c) * plane + col + int64_t(i) * g.nnx])
                                             : 0u);
  };

  float cur[Y + 1][3], nxt[Y + 1][3], raw[Y + 1][3];
  load_layer(z0 - 1, cur);
  load_layer(z0, nxt);
  float fn[Y];
  load_f(z0 - 1, fn);
  unsigned kbn[Y + 1];
  load_kb(z0 - 1, kbn);
  float pend[Y + 1][3];
#pragma unroll
  for (int i = 0; i <= Y; ++i) pend[i][0] = pend[i][1] = pend[i][2] = 0.0f;
  float dsum = 0.0f;

  // The right-hand side and inverse diagonal of node row i, layer c (smoothing
  // and residual modes), requested an element ahead of their use.
  auto load_bd = [&](int i, int c, float (&bv)[3], float (&dv)[3]) {
    const bool ok = c >= 0 && c < g.nnz && ro[i];
    const int64_t d0 = 3 * (int64_t(c) * plane + col + int64_t(i) * g.nnx);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      bv[k] = (MODE != kApply && ok) ? b[d0 + k] : 0.0f;
      dv[k] = (MODE == kSmooth && ok) ? invdiag[d0 + k] : 0.0f;
    }
  };
  // Writes node row i of layer ez from its finished sum ax.
  auto emit = [&](int i, int ez, unsigned kb, const float (&ax)[3], const float (&bv)[3],
                  const float (&dv)[3]) {
    const int64_t d0 = 3 * (int64_t(ez) * plane + col + int64_t(i) * g.nnx);
    float nd = 0.0f;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const int64_t d = d0 + k;
      const bool kk = kn != nullptr ? ((kb >> k) & 1u) != 0u : (kept == nullptr || kept[d] != 0);
      float out;
      if constexpr (MODE == kApply) {
        out = kk ? ax[k] : 0.0f;
        nd = fmaf(cur[i][k], out, nd);
      } else if constexpr (MODE == kResidual) {
        out = kk ? bv[k] - ax[k] : 0.0f;
      } else {
        out = kk ? cur[i][k] + omega * dv[k] * (bv[k] - ax[k]) : 0.0f;
        nd = fmaf(bv[k], out, nd);
      }
      y[d] = out;
    }
    if constexpr (MODE != kResidual) dsum += nd;
  };

#pragma unroll 1
  for (int s = 0; s <= KZ; ++s) {
    const int ez = z0 - 1 + s;
    if (s < KZ) load_layer(ez + 2, raw);
    float f[Y];
    unsigned kb[Y + 1];
#pragma unroll
    for (int j = 0; j < Y; ++j) f[j] = fn[j];
#pragma unroll
    for (int i = 1; i <= Y; ++i) kb[i] = kbn[i];
    if (s < KZ) {
      load_f(ez + 1, fn);
      load_kb(ez + 1, kbn);
    }
    const bool out_z = s >= 1 && ez < g.nnz;
    float bv[3], dv[3];
    load_bd(1, out_z ? ez : -1, bv, dv);
    // x + 1 node values of the element's lower row (cur, nxt layers).
    float c1[3], n1[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      c1[k] = shfl_down(cur[0][k], 1);
      n1[k] = shfl_down(nxt[0][k], 1);
    }
    float C[2][2][3];  // the previous element's +y corners [cx][cz][comp]
#pragma unroll
    for (int j = 0; j < Y; ++j) {
      float c1u[3], n1u[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        c1u[k] = shfl_down(cur[j + 1][k], 1);
        n1u[k] = shfl_down(nxt[j + 1][k], 1);
      }
      // corner c = xb | yb << 1 | zb << 2
      float ux[8] = {cur[j][0], c1[0], cur[j + 1][0], c1u[0], nxt[j][0], n1[0], nxt[j + 1][0], n1u[0]};
      float uy[8] = {cur[j][1], c1[1], cur[j + 1][1], c1u[1], nxt[j][1], n1[1], nxt[j + 1][1], n1u[1]};
      float uz[8] = {cur[j][2], c1[2], cur[j + 1][2], c1u[2], nxt[j][2], n1[2], nxt[j + 1][2], n1u[2]};
      if (f[j] != 0.0f) {
        if constexpr (PK) {
          float2 uxy[8];
#pragma unroll
          for (int c = 0; c < 8; ++c) uxy[c] = make_float2(ux[c], uy[c]);
          modal_apply_xy(mc, f[j], uxy, uz);
#pragma unroll
          for (int c = 0; c < 8; ++c) {
            ux[c] = uxy[c].x;
            uy[c] = uxy[c].y;
          }
        } else {
          modal_apply(mc, f[j], ux, uy, uz);
        }
      } else {
#pragma unroll
        for (int c = 0; c < 8; ++c) ux[c] = uy[c] = uz[c] = 0.0f;
      }
      // Node row j: the previous element's +y corners and this element's -y
      // corners, then the x-combine with the lane below.
      float T[2][2][3];
#pragma unroll
      for (int cx = 0; cx < 2; ++cx)
#pragma unroll
        for (int cz = 0; cz < 2; ++cz) {
          const int c0 = cx | (cz << 2), c1i = cx | 2 | (cz << 2);
          T[cx][cz][0] = j > 0 ? C[cx][cz][0] + ux[c0] : ux[c0];
          T[cx][cz][1] = j > 0 ? C[cx][cz][1] + uy[c0] : uy[c0];
          T[cx][cz][2] = j > 0 ? C[cx][cz][2] + uz[c0] : uz[c0];
          C[cx][cz][0] = ux[c1i];
          C[cx][cz][1] = uy[c1i];
          C[cx][cz][2] = uz[c1i];
        }
      float N[2][3];
#pragma unroll
      for (int cz = 0; cz < 2; ++cz)
#pragma unroll
        for (int k = 0; k < 3; ++k) N[cz][k] = T[0][cz][k] + shfl_up(T[1][cz][k], 1);
      if (j == 0) {
#pragma unroll
        for (int cz = 0; cz < 2; ++cz)
#pragma unroll
          for (int k = 0; k < 3; ++k) xs[s & 1][w][cz * 3 + k][lane] = N[cz][k];
      } else {
        float ax[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          ax[k] = pend[j][k] + N[0][k];
          pend[j][k] = N[1][k];
        }
        if (out_z && ro[j]) emit(j, ez, kb[j], ax, bv, dv);
        load_bd(j + 1, out_z ? ez : -1, bv, dv);
      }
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        c1[k] = c1u[k];
        n1[k] = n1u[k];
      }
    }
    // Node row Y: this thread's top element's +y corners and the next warp's
    // bottom element's -y corners (through shared memory).
    float NY[2][3];
#pragma unroll
    for (int cz = 0; cz < 2; ++cz)
#pragma unroll
      for (int k = 0; k < 3; ++k) NY[cz][k] = C[0][cz][k] + shfl_up(C[1][cz][k], 1);
    __syncthreads();
    if (w < W - 1) {
      float ax[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        ax[k] = pend[Y][k] + (NY[0][k] + xs[s & 1][w + 1][k][lane]);
        pend[Y][k] = NY[1][k] + xs[s & 1][w + 1][3 + k][lane];
      }
      if (out_z && ro[Y]) emit(Y, ez, kb[Y], ax, bv, dv);
    }
#pragma unroll
    for (int i = 0; i <= Y; ++i)
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        cur[i][k] = nxt[i][k];
        nxt[i][k] = raw[i][k];
      }
  }
  if (MODE != kResidual && dot_part != nullptr) {
    const double sum = block_sum(double(dsum));
    if (threadIdx.x == 0)
      dot_part[(int64_t(blockIdx.z) * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x] = sum;
  }
}

// Tile shapes of the column kernel (Y element rows per thread, W warps per CTA)
// and the z-chunk target; the shape is picked per grid (fine_op_col_shape).
struct ColCfg {
  int shape;  // index into kColShapes
  int kz;     // element layers per CTA
};
struct ColShapeDesc {
  int Y, W;
};
constexpr ColShapeDesc kColShapes[] = {{4, 4}, {6, 4}, {3, 4}, {2, 8}};
constexpr int kNumColShapes = 8;  // shapes 4..7: the same tiles with the packed (x, y) arithmetic

static dim3 col_grid(const Grid& g, const ColCfg& c) {
  const ColShapeDesc d = kColShapes[c.shape % 4];
  const int rows = d.W * d.Y - 1;
  return dim3((g.nnx + 29) / 30, (g.nny + rows - 1) / rows, (g.nnz + c.kz - 1) / c.kz);
}

template <class T>
static dim3 pencil_grid(const Grid& g) {
  using P = Pencil<T>;
  return dim3((g.nnx + 30) / 31, (g.nny + P::PY - 2) / (P::PY - 1), (g.nnz + P::KZ - 1) / P::KZ);
}

// Smallest z-chunk the column schedule uses: bounds the partial-sum count.
constexpr int kColMinKz = 8;

int fine_op_blocks(const Grid& g, bool fp64) {
  const dim3 d = fp64 ? pencil_grid<double>(g) : pencil_grid<float>(g);
  int n = int(d.x * d.y * d.z);
  if (!fp64)
    for (int sh = 0; sh < kNumColShapes; ++sh) {
      const dim3 c = col_grid(g, ColCfg{sh, kColMinKz});
      n = std::max(n, int(c.x * c.y * c.z));
    }
  return n;
}

// z-chunk length: chunks of at most `target` element layers that divide the
// node layers evenly (fewest chunks, then the shortest chunk that covers).
static int even_kz(int nnz, int target) {
  const int chunks = std::max(1, (nnz + target - 1) / target);
  return std::max(kColMinKz, (nnz + chunks - 1) / chunks);
}

FineSchedule default_fine_schedule(const Grid& g) {
  FineSchedule s;
  s.kind = FineSchedule::kColumn;
  s.shape = 0;
  s.kz = even_kz(g.nnz, 32);
  return s;
}

int fine_schedule_shapes() { return kNumColShapes; }

bool fine_schedule_valid(const FineSchedule& s) {
  if (s.kind == FineSchedule::kPencil) return true;
  return s.kind == FineSchedule::kColumn && s.shape >= 0 && s.shape < kNumColShapes &&
         s.kz >= kColMinKz && s.kz <= 4096;
}

template <int Y, int W, int MODE, bool PK>
static void launch_col(const Grid& g, const ColCfg& cc, const ModalConsts& c, const float* ef,
                       const uint8_t* kept, const uint8_t* kn, const float* x, const float* b,
                       const float* invdiag, float omega, float* y, double* dot_part,
                       cudaStream_t s) {
  const GridDev gd{g.nx, g.ny, g.nz, g.nnx, g.nny, g.nnz};
  k_fine_op_col<Y, W, MODE, PK><<<col_grid(g, cc), 32 * W, 0, s>>>(
      gd, to_modal<float>(c), cc.kz, ef, kept, kn, x, b, invdiag, omega, y, dot_part);
  TG_LAUNCH_CHECK();
}

template <int MODE>
static void launch_col_shape(const Grid& g, const ColCfg& cc, const ModalConsts& c,
                             const float* ef, const uint8_t* kept, const uint8_t* kn,
                             const float* x, const float* b, const float* invdiag, float omega,
                             float* y, double* dot_part, cudaStream_t s) {
  switch (cc.shape) {
    case 0:
      launch_col<4, 4, MODE, false>(g, cc, c, ef, kept, kn, x, b, invdiag, omega, y, dot_part, s);
      break;
    case 1:
      launch_col<6, 4, MODE, false>(g, cc, c, ef, kept, kn, x, b, invdiag, omega, y, dot_part, s);
      break;
    case 2:
      launch_col<3, 4, MODE, false>(g, cc, c, ef, kept, kn, x, b, invdiag, omega, y, dot_part, s);
      break;
    case 3:
      launch_col<2, 8, MODE, false>(g, cc, c, ef, kept, kn, x, b, invdiag, omega, y, dot_part, s);
      break;
    case 4:
      launch_col<4, 4, MODE, true>(g, cc, c, ef, kept, kn, x, b, invdiag, omega, y, dot_part, s);
      break;
    case 5:
      launch_col<6, 4, MODE, true>(g, cc, c, ef, kept, kn, x, b, invdiag, omega, y, dot_part, s);
      break;
    case 6:
      launch_col<3, 4, MODE, true>(g, cc, c, ef, kept, kn, x, b, invdiag, omega, y, dot_part, s);
      break;
    default:
      launch_col<2, 8, MODE, true>(g, cc, c, ef, kept, kn, x, b, invdiag, omega, y, dot_part, s);
  }
}

template <class T, int MODE>
static void launch_mode(const Grid& g, const ModalConsts& c, const T* ef, const uint8_t* kept,
                        const T* x, const T* b, const T* invdiag, T omega, T* y,
                        double* dot_part, cudaStream_t s) {
  using P = Pencil<T>;
  const GridDev gd{g.nx, g.ny, g.nz, g.nnx, g.nny, g.nnz};
  k_fine_op<T, P::PY, P::KZ, P::MINB, MODE><<<pencil_grid<T>(g), 32 * P::PY, 0, s>>>(
      gd, to_modal<T>(c), ef, kept, x, b, invdiag, omega, y, dot_part);
  TG_LAUNCH_CHECK();
}

template <class T>
void launch_fine_op(int mode, const Grid& g, const ModalConsts& c, const T* ef,
                    const uint8_t* kept, const T* x, const T* b, const T* invdiag, T omega,
                    T* y, double* dot_part, int* nblocks_out, cudaStream_t s,
                    const uint8_t* kn) {
  if constexpr (std::is_same<T, float>::value) {
    launch_fine_op_sched(fine_schedule_for(g, mode), mode, g, c, ef, kept, x, b, invdiag, omega, y,
                         dot_part, nblocks_out, s, kn);
    return;
  }
  if (nblocks_out) {
    const dim3 d = pencil_grid<T>(g);
    *nblocks_out = int(d.x * d.y * d.z);
  }
  switch (mode) {
    case kApply:
      launch_mode<T, kApply>(g, c, ef, kept, x, b, invdiag, omega, y, dot_part, s);
      break;
    case kResidual:
      launch_mode<T, kResidual>(g, c, ef, kept, x, b, invdiag, omega, y, dot_part, s);
      break;
    default:
      launch_mode<T, kSmooth>(g, c, ef, kept, x, b, invdiag, omega, y, dot_part, s);
  }
}

// The FP32 operator under an explicit schedule (the autotuner times candidates
// through this without touching the process-wide table).
void launch_fine_op_sched(const FineSchedule& fs, int mode, const Grid& g, const ModalConsts& c,
                          const float* ef, const uint8_t* kept, const float* x, const float* b,
                          const float* invdiag, float omega, float* y, double* dot_part,
                          int* nblocks_out, cudaStream_t s, const uint8_t* kn) {
  using T = float;
  {
    if (fs.kind == FineSchedule::kColumn) {
      const ColCfg cc{fs.shape, fs.kz};
      if (nblocks_out) {
        const dim3 d = col_grid(g, cc);
        *nblocks_out = int(d.x * d.y * d.z);
      }
      if (mode == kApply)
        launch_col_shape<kApply>(g, cc, c, ef, kept, kn, x, b, invdiag, omega, y, dot_part, s);
      else if (mode == kResidual)
        launch_col_shape<kResidual>(g, cc, c, ef, kept, kn, x, b, invdiag, omega, y, dot_part, s);
      else
        launch_col_shape<kSmooth>(g, cc, c, ef, kept, kn, x, b, invdiag, omega, y, dot_part, s);
      return;
    }
  }
  // The pencil kernel has no fused b . y: its partials come from a dot kernel.
  if (nblocks_out) {
    const dim3 d = pencil_grid<T>(g);
    *nblocks_out = mode == kSmooth && dot_part != nullptr ? kRedBlocks : int(d.x * d.y * d.z);
  }
  switch (mode) {
    case kApply:
      launch_mode<T, kApply>(g, c, ef, kept, x, b, invdiag, omega, y, dot_part, s);
      break;
    case kResidual:
      launch_mode<T, kResidual>(g, c, ef, kept, x, b, invdiag, omega, y, nullptr, s);
      break;
    default:
      launch_mode<T, kSmooth>(g, c, ef, kept, x, b, invdiag, omega, y, nullptr, s);
      if (dot_part != nullptr) launch_dot_partials_f(b, y, g.ndof, dot_part, s);
  }
}

// The FP64 residual y = b - A x evaluated in double-float arithmetic (tg_df.h):
// FP64 inputs and output, about 48 significant bits inside, on the FP32 pipe.
void launch_fine_residual_df(const Grid& g, const ModalConsts& c, const double* ef,
                             const uint8_t* kept, const double* x, const double* b, double* y,
                             cudaStream_t s) {
  using P = Pencil<df>;
  const GridDev gd{g.nx, g.ny, g.nz, g.nnx, g.nny, g.nnz};
  const dim3 grid((g.nnx + 30) / 31, (g.nny + P::PY - 2) / (P::PY - 1), (g.nnz + P::KZ - 1) / P::KZ);
  k_fine_op<double, P::PY, P::KZ, P::MINB, kResidual, false, df><<<grid, 32 * P::PY, 0, s>>>(
      gd, to_modal<df>(c), ef, kept, x, b, nullptr, 0.0, y, nullptr);
  TG_LAUNCH_CHECK();
}

template void launch_fine_op<double>(int, const Grid&, const ModalConsts&, const double*,
                                     const uint8_t*, const double*, const double*,
                                     const double*, double, double*, double*, int*,
                                     cudaStream_t, const uint8_t*);
template void launch_fine_op<float>(int, const Grid&, const ModalConsts&, const float*,
                                    const uint8_t*, const float*, const float*, const float*,
                                    float, float*, double*, int*, cudaStream_t,
                                    const uint8_t*);

// Periodic batched apply: nsys systems on the nx*ny*nz torus; system bi uses
// x/b/y at bi*ndof and the factors / kept mask / inverse diagonal of cell
// bi / nrhs.  dot_part (kApply) receives one partial of x.y per CTA, the CTAs of
// a system contiguous: periodic_op_blocks<T>() per system.
template <class T>
int periodic_op_blocks(int nx, int ny, int nz) {
  using P = Pencil<T>;
  return ((nx + 30) / 31) * ((ny + P::PY - 2) / (P::PY - 1)) * ((nz + P::KZ - 1) / P::KZ);
}
template int periodic_op_blocks<double>(int, int, int);
template int periodic_op_blocks<float>(int, int, int);

template <class T, int MODE>
static void launch_periodic_mode(int nx, int ny, int nz, const ModalConsts& c, const T* ef,
                                 const uint8_t* kept, const T* x, const T* b, const T* invdiag,
                                 T omega, T* y, double* dot_part, int nsys, int nrhs,
                                 cudaStream_t s) {
  using P = Pencil<T>;
  const GridDev gd{nx, ny, nz, nx, ny, nz};
  const int nzc = (nz + P::KZ - 1) / P::KZ;
  const int64_t ndof = 3 * int64_t(nx) * ny * nz, nv = int64_t(nx) * ny * nz;
  // gridDim.z <= 65535: whole cells per launch.
  const int cells_per = std::max(1, 65535 / (nzc * nrhs));
  const int ncell = nsys / nrhs;
  const int nblk = periodic_op_blocks<T>(nx, ny, nz);
  for (int c0 = 0; c0 < ncell; c0 += cells_per) {
    const int nc = std::min(cells_per, ncell - c0);
    const int64_t s0 = int64_t(c0) * nrhs;
    const BatchDev bd{nrhs, nzc, ndof, nv, ndof};
    const dim3 grid((nx + 30) / 31, (ny + P::PY - 2) / (P::PY - 1), nzc * nc * nrhs);
    k_fine_op<T, P::PY, P::KZ, P::MINB, MODE, true><<<grid, 32 * P::PY, 0, s>>>(
        gd, to_modal<T>(c), ef + c0 * nv, kept ? kept + c0 * ndof : nullptr, x + s0 * ndof,
        b ? b + s0 * ndof : nullptr, invdiag ? invdiag + c0 * ndof : nullptr, omega,
        y + s0 * ndof, dot_part ? dot_part + s0 * nblk : nullptr, bd);
    TG_LAUNCH_CHECK();
  }
}

template <class T>
void launch_periodic_op(int mode, int nx, int ny, int nz, const ModalConsts& c, const T* ef,
                        const uint8_t* kept, const T* x, const T* b, const T* invdiag, T omega,
                        T* y, double* dot_part, int nsys, int nrhs, cudaStream_t s) {
  if (mode == kApply)
    launch_periodic_mode<T, kApply>(nx, ny, nz, c, ef, kept, x, b, invdiag, omega, y, dot_part,
                                    nsys, nrhs, s);
  else if (mode == kResidual)
    launch_periodic_mode<T, kResidual>(nx, ny, nz, c, ef, kept, x, b, invdiag, omega, y,
                                       dot_part, nsys, nrhs, s);
  else
    launch_periodic_mode<T, kSmooth>(nx, ny, nz, c, ef, kept, x, b, invdiag, omega, y, dot_part,
                                     nsys, nrhs, s);
}
template void launch_periodic_op<double>(int, int, int, int, const ModalConsts&, const double*,
                                         const uint8_t*, const double*, const double*,
                                         const double*, double, double*, double*, int, int,
                                         cudaStream_t);
template void launch_periodic_op<float>(int, int, int, int, const ModalConsts&, const float*,
                                        const uint8_t*, const float*, const float*, const float*,
                                        float, float*, double*, int, int, cudaStream_t);

// diag(A) at every DOF = kdiag * (sum of the adjacent element factors), summed
// in a fixed element order; invdiag = 1/diag on kept DOFs, 0 elsewhere
// (matfree.cpp:757-833 accumulates factor_e * Ke(r,r)).
__global__ void k_fine_invdiag(GridDev g, double kdiag, const double* __restrict__ ef,
                               const uint8_t* __restrict__ kept, double* __restrict__ invdiag) {
  const int64_t n = int64_t(g.nnx) * g.nny * g.nnz;
  for (int64_t node = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; node < n;
       node += int64_t(gridDim.x) * blockDim.x) {
    const int a = int(node % g.nnx);
    const int bb = int((node / g.nnx) % g.nny);
    const int c = int(node / (int64_t(g.nnx) * g.nny));
    double s = 0.0;
    for (int dz = -1; dz <= 0; ++dz)
      for (int dy = -1; dy <= 0; ++dy)
        for (int dx = -1; dx <= 0; ++dx) {
          const int i = a + dx, j = bb + dy, k = c + dz;
          if (i < 0 || i >= g.nx || j < 0 || j >= g.ny || k < 0 || k >= g.nz) continue;
          s += ef[(int64_t(k) * g.ny + j) * g.nx + i];
        }
    const double dg = kdiag * s;
    for (int comp = 0; comp < 3; ++comp) {
      const int64_t d = 3 * node + comp;
      invdiag[d] = (kept[d] && dg > 0.0) ? 1.0 / dg : 0.0;
    }
  }
}

void launch_fine_invdiag(const Grid& g, double kdiag, const double* ef, const uint8_t* kept,
                         double* invdiag, cudaStream_t s) {
  const GridDev gd{g.nx, g.ny, g.nz, g.nnx, g.nny, g.nnz};
  const int64_t blocks = std::min<int64_t>((g.nnodes + 255) / 256, 152 * 16);
  k_fine_invdiag<<<int(blocks), 256, 0, s>>>(gd, kdiag, ef, kept, invdiag);
  TG_LAUNCH_CHECK();
}

}  // namespace tg
