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
// Scheduling: one CTA owns a brick of BX x BY x BZ nodes.  It stages the
// (BX+2)(BY+2)(BZ+2) node values it needs in shared memory, evaluates every
// element adjacent to an owned node (a one-element halo is recomputed by the
// neighbouring brick), and accumulates element outputs into shared memory in
// eight corner sub-steps: in sub-step k every element adds its corner-k output,
// so no two writers meet and the per-node summation order is fixed -- the apply
// is deterministic run to run without atomics.
#include <cuda_runtime.h>

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

template <class T>
ModalT<T> to_modal(const ModalConsts& c) {
  ModalT<T> m;
  m.L0 = T(c.L[0]);
  m.L1 = T(c.L[1]);
  m.M0 = T(c.M[0]);
  m.M1 = T(c.M[1]);
  m.M02 = T(2.0 * c.M[0]);
  m.M12 = T(2.0 * c.M[1]);
  m.LM2 = T(c.L[2] + 4.0 * c.M[2]);
  return m;
}

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
    gx[1] = Ltr + M02 * ux[1];
    gy[2] = Ltr + M02 * uy[2];
    gz[4] = Ltr + M02 * uz[4];
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
    gy[3] = Ltr + M12 * uy[3];
    gz[3] = t;
    gx[5] = M1 * ux[5];
    gy[5] = t;
    gz[5] = Ltr + M12 * uz[5];
  }
  {
    const T Ltr = L1 * (ux[3] + uz[6]);  // T = {y}: rows x (mode 3), z (mode 6)
    const T t = M1 * (uz[3] + ux[6]);
    gx[3] += Ltr + M12 * ux[3];
    gy[3] += M1 * uy[3];
    gz[3] += t;
    gx[6] = t;
    gy[6] = M1 * uy[6];
    gz[6] = Ltr + M12 * uz[6];
  }
  {
    const T Ltr = L1 * (ux[5] + uy[6]);  // T = {z}: rows x (mode 5), y (mode 6)
    const T t = M1 * (uy[5] + ux[6]);
    gx[5] += Ltr + M12 * ux[5];
    gy[5] += t;
    gz[5] += M1 * uz[5];
    gx[6] += t;
    gy[6] += Ltr + M12 * uy[6];
    gz[6] += M1 * uz[6];
  }
  // |T| = 2: the trilinear mode.
  gx[7] = LM2 * ux[7];
  gy[7] = LM2 * uy[7];
  gz[7] = LM2 * uz[7];
  gx[0] = gy[0] = gz[0] = T(0);
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

struct GridDev {
  int nx, ny, nz, nnx, nny, nnz;
};

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

template <class T, int BX, int BY, int BZ, int NT, int MODE>
__global__ void __launch_bounds__(NT) k_fine_op(GridDev g, ModalT<T> mc,
                                                const T* __restrict__ ef,
                                                const uint8_t* __restrict__ kept,
                                                const T* __restrict__ x, const T* __restrict__ b,
                                                const T* __restrict__ invdiag, T omega,
                                                T* __restrict__ y, double* __restrict__ dot_part) {
  constexpr int TX = BX + 2, TY = BY + 2, TZ = BZ + 2, TN = TX * TY * TZ;
  constexpr int EX = BX + 1, EY = BY + 1, EZ = BZ + 1, EN = EX * EY * EZ;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* xs = reinterpret_cast<T*>(smem_raw);
  T* ys = xs + 3 * TN;
  const int n0x = blockIdx.x * BX, n0y = blockIdx.y * BY, n0z = blockIdx.z * BZ;

  // Stage the node tile [n0-1, n0+B] (zeros outside the grid) and clear ys.
  for (int t3 = threadIdx.x; t3 < 3 * TN; t3 += NT) {
    const int t = t3 / 3, c = t3 - 3 * t;
    const int lx = t % TX, ly = (t / TX) % TY, lz = t / (TX * TY);
    const int gx = n0x - 1 + lx, gy = n0y - 1 + ly, gz = n0z - 1 + lz;
    T v = T(0);
    if (gx >= 0 && gx < g.nnx && gy >= 0 && gy < g.nny && gz >= 0 && gz < g.nnz)
      v = x[3 * ((int64_t(gz) * g.nny + gy) * g.nnx + gx) + c];
    xs[t3] = v;
    ys[t3] = T(0);
  }
  __syncthreads();

  for (int base = 0; base < EN; base += NT) {
    const int le = base + threadIdx.x;
    bool active = false;
    int ex = 0, ey = 0, ez = 0;
    T ux[8], uy[8], uz[8];
    if (le < EN) {
      ex = le % EX;
      ey = (le / EX) % EY;
      ez = le / (EX * EY);
      const int gex = n0x - 1 + ex, gey = n0y - 1 + ey, gez = n0z - 1 + ez;
      if (gex >= 0 && gex < g.nx && gey >= 0 && gey < g.ny && gez >= 0 && gez < g.nz) {
        const T f = ef[(int64_t(gez) * g.ny + gey) * g.nx + gex];
        if (f != T(0)) {
          active = true;
#pragma unroll
          for (int k = 0; k < 8; ++k) {
            const int tl = ((ez + (k >> 2)) * TY + (ey + ((k >> 1) & 1))) * TX + ex + (k & 1);
            ux[k] = xs[3 * tl];
            uy[k] = xs[3 * tl + 1];
            uz[k] = xs[3 * tl + 2];
          }
          modal_apply(mc, f, ux, uy, uz);
        }
      }
    }
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      if (active) {
        const int tl = ((ez + (k >> 2)) * TY + (ey + ((k >> 1) & 1))) * TX + ex + (k & 1);
        ys[3 * tl] += ux[k];
        ys[3 * tl + 1] += uy[k];
        ys[3 * tl + 2] += uz[k];
      }
      __syncthreads();
    }
  }

  double dsum = 0.0;
  for (int t3 = threadIdx.x; t3 < 3 * BX * BY * BZ; t3 += NT) {
    const int t = t3 / 3, c = t3 - 3 * t;
    const int ox = t % BX, oy = (t / BX) % BY, oz = t / (BX * BY);
    const int gx = n0x + ox, gy = n0y + oy, gz = n0z + oz;
    if (gx >= g.nnx || gy >= g.nny || gz >= g.nnz) continue;
    const int tl = ((oz + 1) * TY + (oy + 1)) * TX + ox + 1;
    const int64_t d = 3 * ((int64_t(gz) * g.nny + gy) * g.nnx + gx) + c;
    const bool k = kept == nullptr || kept[d] != 0;
    const T ax = ys[3 * tl + c];
    T out;
    if (MODE == kApply) {
      out = k ? ax : T(0);
      dsum += double(xs[3 * tl + c]) * double(out);
    } else if (MODE == kResidual) {
      out = k ? T(b[d] - ax) : T(0);
    } else {
      out = k ? T(xs[3 * tl + c] + omega * invdiag[d] * (b[d] - ax)) : T(0);
    }
    y[d] = out;
  }
  if (MODE == kApply && dot_part != nullptr) {
    const double s = block_sum(dsum);
    if (threadIdx.x == 0)
      dot_part[(int64_t(blockIdx.z) * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x] = s;
  }
}

template <class T>
struct Brick;
template <>
struct Brick<double> {
  static constexpr int BX = 8, BY = 8, BZ = 8, NT = 256;
};
template <>
struct Brick<float> {
  static constexpr int BX = 16, BY = 8, BZ = 8, NT = 512;
};

int fine_op_blocks(const Grid& g, bool fp64) {
  const int bx = fp64 ? Brick<double>::BX : Brick<float>::BX;
  const int by = fp64 ? Brick<double>::BY : Brick<float>::BY;
  const int bz = fp64 ? Brick<double>::BZ : Brick<float>::BZ;
  return ((g.nnx + bx - 1) / bx) * ((g.nny + by - 1) / by) * ((g.nnz + bz - 1) / bz);
}

template <class T, int MODE>
static void launch_mode(const Grid& g, const ModalConsts& c, const T* ef, const uint8_t* kept,
                        const T* x, const T* b, const T* invdiag, T omega, T* y,
                        double* dot_part, cudaStream_t s) {
  using B = Brick<T>;
  constexpr int TN = (B::BX + 2) * (B::BY + 2) * (B::BZ + 2);
  constexpr size_t smem = 2 * 3 * TN * sizeof(T);
  auto kern = k_fine_op<T, B::BX, B::BY, B::BZ, B::NT, MODE>;
  static bool configured = false;
  if (!configured) {
    TG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    configured = true;
  }
  const dim3 grid((g.nnx + B::BX - 1) / B::BX, (g.nny + B::BY - 1) / B::BY,
                  (g.nnz + B::BZ - 1) / B::BZ);
  const GridDev gd{g.nx, g.ny, g.nz, g.nnx, g.nny, g.nnz};
  kern<<<grid, B::NT, smem, s>>>(gd, to_modal<T>(c), ef, kept, x, b, invdiag, omega, y, dot_part);
  TG_LAUNCH_CHECK();
}

template <class T>
void launch_fine_op(int mode, const Grid& g, const ModalConsts& c, const T* ef,
                    const uint8_t* kept, const T* x, const T* b, const T* invdiag, T omega,
                    T* y, double* dot_part, int* nblocks_out, cudaStream_t s) {
  if (nblocks_out) *nblocks_out = fine_op_blocks(g, sizeof(T) == 8);
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

template void launch_fine_op<double>(int, const Grid&, const ModalConsts&, const double*,
                                     const uint8_t*, const double*, const double*,
                                     const double*, double, double*, double*, int*,
                                     cudaStream_t);
template void launch_fine_op<float>(int, const Grid&, const ModalConsts&, const float*,
                                    const uint8_t*, const float*, const float*, const float*,
                                    float, float*, double*, int*, cudaStream_t);

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
