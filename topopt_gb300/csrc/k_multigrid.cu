// k_multigrid.cu -- geometric multigrid on the voxel hierarchy.
//
// Reference counterparts (core/src/fea/multigrid.cpp):
//   axis_weights           :494-505   trilinear vertex stencil 1 | 1/2,1/2
//   coarse active DOFs     :1387-1403 active iff the coincident fine DOF is
//   P0 and A1 = P0^T A0 P0 :1408-1446, galerkin_a1_from_prolong :1543-1899
//   levels 2.. (Galerkin)  :557-697 (build_hierarchy)
//   jacobi_sweep, v_cycle  :780-817, mf_jacobi_sweep / mf_v_cycle :1128-1160
//   coarsest direct solve  SimplicialLDLT :690-695 -> here a dense Cholesky
//
// Coarse operators are Galerkin, formed element by element: a coarse element's
// 24x24 matrix is the sum over its (up to) eight children of W^T K_child W, with
// W the trilinear interpolation from the parent's 8 nodes to the child's 8
// nodes.  Because P restricted to an element is exactly that local W, the
// assembled sum equals P^T A P -- including the masks: rows and columns of
// inactive DOFs are zeroed on both sides, as the reference drops them from P.
// Odd axes are handled by ceil-halving the element extents; a coarse node whose
// coincident fine node lies beyond the grid is inactive, which reproduces the
// reference's index-space padding (multigrid.cpp:391-459).
//
// Coarse levels are applied as assembled 27-point node stencils.  The operator
// is symmetric, so only the self block and the 13 "forward" neighbour blocks
// (positive linear offset) are stored, as structure of arrays A[126][nnodes]
// (entry (j*3 + c1)*3 + c2 for block j): a thread per node reads its own rows
// coalesced and the backward blocks, transposed, from the neighbour's rows.
// Half the bytes of the full 243-entry stencil, the bound of the coarse apply.
#include <cuda_runtime.h>

#include "tg_internal.h"
#include "tg_multigrid.h"

#include <algorithm>
#include <atomic>

namespace tg {

namespace {
constexpr int kThreads = 256;

int nblk(int64_t n, int t = kThreads) {
  const int64_t b = (n + t - 1) / t;
  return int(b < 152 * 64 ? (b > 0 ? b : 1) : 152 * 64);
}

// Coordinates (a, b, c) of linear node index n of a level: 32-bit unsigned
// division whenever the index fits (every coarse level; a 64-bit division is a
// long dependent instruction sequence that small, latency-bound kernels pay on
// every item).
__device__ __forceinline__ void node_abc(const MgDims& d, int64_t n, int& a, int& b, int& c) {
  if (n <= int64_t(0xffffffffu)) {
    const unsigned un = unsigned(n), nx = unsigned(d.nnx), ny = unsigned(d.nny);
    const unsigned q = un / nx, r = q / ny;
    a = int(un - q * nx);
    b = int(q - r * ny);
    c = int(r);
  } else {
    a = int(n % d.nnx);
    b = int((n / d.nnx) % d.nny);
    c = int(n / (int64_t(d.nnx) * d.nny));
  }
}

// Local corner index -> offsets; corners in Walsh bit order (x | y<<1 | z<<2).
__device__ __forceinline__ int cx(int c) { return c & 1; }
__device__ __forceinline__ int cy(int c) { return (c >> 1) & 1; }
__device__ __forceinline__ int cz(int c) { return c >> 2; }

// v[3*corner + comp] <- sum_sc v[3*sc + comp] * prod_a M_a[sc_a][t_a] for every
// parent corner t: three 2x2 passes over the corner bits (x, y, z).
template <class T>
__device__ __forceinline__ void kron_map(const T (&mw)[3][4], T (&v)[24]) {
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const int bit = 1 << a;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      if (i & bit) continue;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const T lo = v[3 * i + c], hi = v[3 * (i | bit) + c];
        v[3 * i + c] = mw[a][0] * lo + mw[a][2] * hi;
        v[3 * (i | bit) + c] = mw[a][1] * lo + mw[a][3] * hi;
      }
    }
  }
}

// One warp per coarse element; lane c < 24 owns column c of the coarse element
// matrix (rows in corner-bit order, row = 3*corner + comp).  For every child,
// X = S W (lane r = row r of S) then Y += W^T X (lane c = column c), with the
// sparsity pattern of W uniform across the warp.  S is the child's matrix:
// level 1 -- f * Ke with inactive fine DOFs zeroed (or the precomputed
// G_c = W_c^T Ke W_c times f when all 24 are active); deeper levels -- the stored,
// already masked, child element matrix.  Rows/cols of inactive coarse DOFs are
// zeroed at the end.
// With skip set, level 1's elements with skip[ce] < 0 are left to
// k_galerkin1_fast.
template <class T, bool LEVEL1>
__global__ void __launch_bounds__(128) k_galerkin(MgDims fd, MgDims cd, const T* __restrict__ ef,
                                                  const uint8_t* __restrict__ fact,
                                                  const uint8_t* __restrict__ cact,
                                                  const T* __restrict__ Ke,
                                                  const T* __restrict__ G,
                                                  const T* __restrict__ Kf,
                                                  T* __restrict__ Kc,
                                                  const int* __restrict__ skip) {
  constexpr int NW = 4;
  constexpr int LD = 25;  // padded row stride: row and column walks are bank-conflict free
  // Level 1 in FP32: the 8 child blocks G_c live in shared memory (18 KB per CTA).
  constexpr bool kSmemG = LEVEL1 && sizeof(T) == 4;
  __shared__ T sS[NW][24 * LD];
  __shared__ T sX[NW][24 * LD];
  __shared__ T sG[kSmemG ? 8 * 576 : 1];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  T* S = sS[warp];
  T* X = sX[warp];
  if (kSmemG) {
    for (int e = threadIdx.x; e < 8 * 576; e += blockDim.x) sG[e] = G[e];
    __syncthreads();
    G = sG;
  }
  const int64_t nce = int64_t(cd.ex) * cd.ey * cd.ez;
  for (int64_t ce = blockIdx.x * int64_t(NW) + warp; ce < nce; ce += int64_t(gridDim.x) * NW) {
    if (skip != nullptr && skip[ce] < 0) continue;  // warp-uniform
    const int I = int(ce % cd.ex), J = int((ce / cd.ex) % cd.ey),
              K = int(ce / (int64_t(cd.ex) * cd.ey));
    const int hm = cd.align ? ((2 * I + 1 == fd.ex) | ((2 * J + 1 == fd.ey) << 1) |
                               ((2 * K + 1 == fd.ez) << 2))
                            : 0;
    T acc[24];
#pragma unroll
    for (int r = 0; r < 24; ++r) acc[r] = T(0);
    // Level 1: the children's moduli (lane ch holds child ch's) and this lane's
    // kept bit of every child (bit ch), all requested before the child loop.
    T f_lane = T(0);
    unsigned int kept_bits = 0;
    if (LEVEL1) {
      if (lane < 8) {
        const int fi = 2 * I + cx(lane), fj = 2 * J + cy(lane), fk = 2 * K + cz(lane);
        if (fi < fd.ex && fj < fd.ey && fk < fd.ez)
          f_lane = ef[(int64_t(fk) * fd.ey + fj) * fd.ex + fi];
      }
      if (lane < 24) {
        const int c = lane / 3, comp = lane % 3;
#pragma unroll
        for (int ch = 0; ch < 8; ++ch) {
          const int fi = 2 * I + cx(ch), fj = 2 * J + cy(ch), fk = 2 * K + cz(ch);
          if (fi >= fd.ex || fj >= fd.ey || fk >= fd.ez) continue;
          const int64_t node =
              (int64_t(fk + cz(c)) * fd.nny + (fj + cy(c))) * fd.nnx + (fi + cx(c));
          if (fact[3 * node + comp]) kept_bits |= 1u << ch;
        }
      }
    }
    for (int ch = 0; ch < 8; ++ch) {
      const int fi = 2 * I + cx(ch), fj = 2 * J + cy(ch), fk = 2 * K + cz(ch);
      if (fi >= fd.ex || fj >= fd.ey || fk >= fd.ez) continue;
      const int64_t fe = (int64_t(fk) * fd.ey + fj) * fd.ex + fi;
      T f = T(1);
      unsigned int m = 0xffffffu;
      if (LEVEL1) {
        f = __shfl_sync(0xffffffffu, f_lane, ch);
        if (f == T(0)) continue;
        m = __reduce_or_sync(0xffffffffu, ((kept_bits >> ch) & 1u) << lane);
        if (m == 0xffffffu && hm == 0) {
          if (lane < 24)
#pragma unroll
            for (int r = 0; r < 24; ++r) acc[r] += f * G[ch * 576 + r * 24 + lane];
          continue;
        }
        for (int e = lane; e < 576; e += 32) {
          const int r = e / 24, c2 = e % 24;
          S[r * LD + c2] = ((m >> r) & 1u) && ((m >> c2) & 1u) ? f * Ke[e] : T(0);
        }
      } else {
        for (int e = lane; e < 576; e += 32) S[(e / 24) * LD + e % 24] = Kf[fe * 576 + e];
      }
      __syncwarp();
      // W = W_x (x) W_y (x) W_z on the corner index (times I3 on components):
      // per axis a 2x2 map from the child's sub-corner bit to the parent's
      // corner bit -- [[1,0],[1/2,1/2]] for child bit 0, [[1/2,1/2],[0,1]] for
      // child bit 1, the identity on an aligned half element.  X = S W and
      // Y += W^T X are three 2x2 passes each instead of a dense 8x8 product.
      T mw[3][4];  // per axis: M[sc][t] as {m00, m01, m10, m11}; warp-uniform
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        const bool half = (hm >> a) & 1, hi = (ch >> a) & 1;
        mw[a][0] = half ? T(1) : (hi ? T(0.5) : T(1));
        mw[a][1] = half ? T(0) : (hi ? T(0.5) : T(0));
        mw[a][2] = half ? T(0) : (hi ? T(0) : T(0.5));
        mw[a][3] = half ? T(1) : (hi ? T(1) : T(0.5));
      }
      if (lane < 24) {  // X = S W: lane = row
        T v[24];
#pragma unroll
        for (int j = 0; j < 24; ++j) v[j] = S[lane * LD + j];
        kron_map(mw, v);
#pragma unroll
        for (int j = 0; j < 24; ++j) X[lane * LD + j] = v[j];
      }
      __syncwarp();
      if (lane < 24) {  // Y += W^T X: lane = column
        T v[24];
#pragma unroll
        for (int j = 0; j < 24; ++j) v[j] = X[j * LD + lane];
        kron_map(mw, v);
#pragma unroll
        for (int j = 0; j < 24; ++j) acc[j] += v[j];
      }
      __syncwarp();
    }
    unsigned int cm = 0;
    if (lane < 24) {
      const int c = lane / 3, comp = lane % 3;
      const int64_t node = (int64_t(K + cz(c)) * cd.nny + (J + cy(c))) * cd.nnx + (I + cx(c));
      if (cact[3 * node + comp]) cm = 1u << lane;
    }
    cm = __reduce_or_sync(0xffffffffu, cm);
    if (lane < 24) {
      const bool colk = (cm >> lane) & 1u;
#pragma unroll
      for (int r = 0; r < 24; ++r) Kc[ce * 576 + r * 24 + lane] = (colk && ((cm >> r) & 1u)) ? acc[r] : T(0);
    }
  }
}

// Node stencil from the element matrices around each node: the self block and
// the forward blocks only.  Entry index q = (j*3 + c1)*3 + c2 with
// j = d - 13, d = (dz+1)*9 + (dy+1)*3 + (dx+1) >= 13.  With A null only the
// inverse diagonal is formed (the self block), from the same sums.
template <class T>
__global__ void k_assemble_stencil(MgDims d, const T* __restrict__ Kel,
                                   const uint8_t* __restrict__ act, T* __restrict__ A,
                                   T* __restrict__ invdiag) {
  const int64_t nn = int64_t(d.nnx) * d.nny * d.nnz;
  for (int64_t n = blockIdx.x * int64_t(kThreads) + threadIdx.x; n < nn;
       n += int64_t(gridDim.x) * kThreads) {
    int a, b, c;
    node_abc(d, n, a, b, c);
    bool ra[3];
    for (int k = 0; k < 3; ++k) ra[k] = act[3 * n + k] != 0;
    for (int dz = -1; dz <= 1; ++dz)
      for (int dy = -1; dy <= 1; ++dy)
        for (int dx = -1; dx <= 1; ++dx) {
          const int di = ((dz + 1) * 3 + (dy + 1)) * 3 + (dx + 1);
          if (di < 13) continue;  // backward blocks: the neighbour's forward block, transposed
          if (A == nullptr && di != 13) continue;
          const int j = di - 13;
          T blk[9];
#pragma unroll
          for (int k = 0; k < 9; ++k) blk[k] = T(0);
          // Elements containing both n and n+d: offsets ox in {-1,0} with the
          // node at corner (-ox) and the neighbour at corner (-ox + dx) in [0,1].
          for (int oz = -1; oz <= 0; ++oz) {
            const int lz = -oz, mz = lz + dz;
            if (mz < 0 || mz > 1) continue;
            for (int oy = -1; oy <= 0; ++oy) {
              const int ly = -oy, my = ly + dy;
              if (my < 0 || my > 1) continue;
              for (int ox = -1; ox <= 0; ++ox) {
                const int lx = -ox, mx = lx + dx;
                if (mx < 0 || mx > 1) continue;
                const int ei = a + ox, ej = b + oy, ek = c + oz;
                if (ei < 0 || ei >= d.ex || ej < 0 || ej >= d.ey || ek < 0 || ek >= d.ez) continue;
                const int64_t e = (int64_t(ek) * d.ey + ej) * d.ex + ei;
                const int ln = lx | (ly << 1) | (lz << 2), lm = mx | (my << 1) | (mz << 2);
                const T* Ke = Kel + e * 576;
#pragma unroll
                for (int c1 = 0; c1 < 3; ++c1)
#pragma unroll
                  for (int c2 = 0; c2 < 3; ++c2) blk[c1 * 3 + c2] += Ke[(3 * ln + c1) * 24 + 3 * lm + c2];
              }
            }
          }
          if (A != nullptr)
#pragma unroll
            for (int c1 = 0; c1 < 3; ++c1)
#pragma unroll
              for (int c2 = 0; c2 < 3; ++c2)
                A[int64_t(j * 9 + c1 * 3 + c2) * nn + n] = ra[c1] ? blk[c1 * 3 + c2] : T(0);
          if (j == 0)
            for (int k = 0; k < 3; ++k) {
              const T dg = blk[k * 3 + k];
              invdiag[3 * n + k] = (ra[k] && dg > T(0)) ? T(1) / dg : T(0);
            }
        }
  }
}

template <class T>
__global__ void k_to_float(const double* __restrict__ s, T* __restrict__ d, int64_t n) {
  for (int64_t i = blockIdx.x * int64_t(kThreads) + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * kThreads)
    d[i] = T(s[i]);
}

// Stencil operator: y = A x / b - A x / x + w D^-1 (b - A x), masked by act.
// A thread per (node, output component r): row r of every 3x3 block.  Forward
// block j of node n couples n to n + off_j; the backward coupling of n to
// n - off_j is the forward block j of node n - off_j, transposed (its column r).
// Three threads per node keep the per-thread register count low and the number
// of independent coefficient loads in flight high: the kernel streams the
// stencil once from HBM (the backward re-reads hit L2) and is bound by how many
// of those loads are outstanding.  Out-of-grid neighbours are predicated (the
// stored forward block of a node whose neighbour lies outside the grid is zero,
// and the backward term is selected away).  Per output the terms are summed in
// the fixed order of stencil_row.
// Loads of vectors another CTA may have written earlier in the same launch (the
// fused coarse V-cycle) go through L2; elsewhere plain loads.
template <class T, bool COH>
__device__ __forceinline__ T vload(const T* p) {
  if constexpr (COH)
    return __ldcg(p);
  else
    return *p;
}

// Chebyshev direction update c0 * d_prev + c1 * res with one explicit rounding
// pattern (the product c1 * res rounded, then one fused multiply-add), so every
// kernel that takes the step produces the same bits.
__device__ __forceinline__ float cheb_dir(float c0, float dprev, float c1, float res) {
  return __fmaf_rn(c0, dprev, __fmul_rn(c1, res));
}
__device__ __forceinline__ double cheb_dir(double c0, double dprev, double c1, double res) {
  return __fma_rn(c0, dprev, __dmul_rn(c1, res));
}

// u = a0 x0 + a1 x1 + a2 x2 with one rounding pattern (a product, then two
// fused multiply-adds) in every kernel that evaluates a stencil term.
__device__ __forceinline__ float dot3(float a0, float x0, float a1, float x1, float a2, float x2) {
  return __fmaf_rn(a2, x2, __fmaf_rn(a1, x1, __fmul_rn(a0, x0)));
}
__device__ __forceinline__ double dot3(double a0, double x0, double a1, double x1, double a2,
                                       double x2) {
  return __fma_rn(a2, x2, __fma_rn(a1, x1, __dmul_rn(a0, x0)));
}

// Part `part` (0..3) of row r of node (a, bb, c) of a stored symmetric stencil
// times x.  The row is the self block (term 0) plus, for j = 1..13, forward
// block j (neighbour n + off_j) and the transposed forward block of neighbour
// n - off_j; part q sums the terms j = q, q + 4, ... in increasing j (part 0
// starts from the self term), and the row is ((p0 + p1) + p2) + p3.  Four
// parts let four threads share a row on the small levels, where a row's ~160
// loads in one thread are a chain of dependent memory round trips.
template <class T, bool COH>
__device__ __forceinline__ T stencil_part(const MgDims& d, const T* __restrict__ A, const T* x,
                                          int a, int bb, int c, int r, int part) {
  const int64_t nn = int64_t(d.nnx) * d.nny * d.nnz;
  const int64_t sy = d.nnx, sz = int64_t(d.nnx) * d.nny;
  const int64_t n = c * sz + bb * sy + a;
  const T* An = A + n + int64_t(3 * r) * nn;  // row r of the self block
  T s = T(0);
  if (part == 0)
    s = dot3(An[0], vload<T, COH>(x + 3 * n), An[nn], vload<T, COH>(x + 3 * n + 1), An[2 * nn],
             vload<T, COH>(x + 3 * n + 2));
#pragma unroll
  for (int j = 1; j < 14; ++j) {
    if ((j & 3) != part) continue;
    const int di = 13 + j;
    const int dx = di % 3 - 1, dy = (di / 3) % 3 - 1, dz = di / 9 - 1;
    const int64_t off = dz * sz + dy * sy + dx;
    const bool fin = (a + dx) < d.nnx && (a + dx) >= 0 && (bb + dy) < d.nny && (bb + dy) >= 0 &&
                     (c + dz) < d.nnz;
    const bool bin = (a - dx) >= 0 && (a - dx) < d.nnx && (bb - dy) >= 0 && (bb - dy) < d.nny &&
                     (c - dz) >= 0;
    const int64_t m = fin ? n + off : n;
    const int64_t p = bin ? n - off : n;
    const T* Af = An + int64_t(j * 9) * nn;
    const T* Ab = A + int64_t(j * 9 + r) * nn + p;
    const T u = dot3(Af[0], vload<T, COH>(x + 3 * m), Af[nn], vload<T, COH>(x + 3 * m + 1),
                     Af[2 * nn], vload<T, COH>(x + 3 * m + 2));
    const T v = dot3(Ab[0], vload<T, COH>(x + 3 * p), Ab[3 * nn], vload<T, COH>(x + 3 * p + 1),
                     Ab[6 * nn], vload<T, COH>(x + 3 * p + 2));
    s += fin ? u : T(0);
    s += bin ? v : T(0);
  }
  return s;
}

// Row r of node (a, bb, c) of the stencil times x: the four parts in order.
template <class T, bool COH>
__device__ __forceinline__ T stencil_row(const MgDims& d, const T* __restrict__ A, const T* x,
                                         int a, int bb, int c, int r) {
  T p[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) p[q] = stencil_part<T, COH>(d, A, x, a, bb, c, r, q);
  return ((p[0] + p[1]) + p[2]) + p[3];
}

// The per-DOF update of the stencil kernels from the row sum s, in one
// rounding pattern: kApply s, kResidual b - s, kSmooth x + (omega dinv)(b - s),
// kCheb the Chebyshev step (direction dprev of the previous step, coefficients
// of the level's table); inactive DOFs 0 (and a zero direction).
template <class T, int MODE>
__device__ __forceinline__ T stencil_update(bool active, T s, T xv, T bv, T dv, T omega,
                                            const float* cf, int step, T dprev, T& dnew) {
  dnew = T(0);
  if (!active) return T(0);
  if (MODE == kApply) return s;
  if (MODE == kResidual) return bv - s;
  if (MODE == kCheb) {
    // Chebyshev step (Saad, Iterative Methods, Alg. 12.1): d_k = rho_k rho_{k-1}
    // d_{k-1} + (2 rho_k / delta) D^-1 (b - A x_k), d_0 = D^-1 (b - A x_0) / theta,
    // x_{k+1} = x_k + d_k.
    const T res = dv * (bv - s);
    dnew = step == 0 ? T(cf[0]) * res : cheb_dir(T(cf[2 * step]), dprev, T(cf[2 * step + 1]), res);
    return xv + dnew;
  }
  if constexpr (sizeof(T) == 4)
    return __fmaf_rn(__fmul_rn(omega, dv), __fsub_rn(bv, s), xv);
  else
    return __fma_rn(__dmul_rn(omega, dv), __dsub_rn(bv, s), xv);
}

constexpr int kStencilThreads = 192;

template <class T, int MODE>
__global__ void __launch_bounds__(kStencilThreads) k_stencil_op(MgDims d, const T* __restrict__ A,
                                                    const uint8_t* __restrict__ act,
                                                    const T* __restrict__ x,
                                                    const T* __restrict__ b,
                                                    const T* __restrict__ invdiag, T omega,
                                                    T* __restrict__ y, ChebStep ch) {
  // 192 threads: two chunks of 32 consecutive nodes (in x-fastest order, across
  // row ends) x 3 components, one component per warp, so a warp's stencil and
  // vector reads are coalesced and no lane idles at the odd row lengths
  // (2^k + 1 nodes) of the coarse levels.
  const int64_t it = blockIdx.x * int64_t(kStencilThreads) + threadIdx.x;
  const int64_t n = (it / 96) * 32 + (it & 31);
  const int r = int((it / 32) % 3);
  if (n >= int64_t(d.nnx) * d.nny * d.nnz) return;
  int a, bb, c;
  node_abc(d, n, a, bb, c);
  const T s = stencil_row<T, false>(d, A, x, a, bb, c, r);
  const int64_t dof = 3 * n + r;
  T* dir = static_cast<T*>(ch.dir_);
  const bool ac = act[dof] != 0;
  T dnew;
  const T out = stencil_update<T, MODE>(
      ac, s, (MODE == kSmooth || MODE == kCheb) ? x[dof] : T(0), MODE != kApply ? b[dof] : T(0),
      (MODE == kSmooth || MODE == kCheb) ? invdiag[dof] : T(0), omega, ch.coef, ch.step,
      (MODE == kCheb && ch.step > 0 && ac) ? dir[dof] : T(0), dnew);
  if (MODE == kCheb) dir[dof] = dnew;
  y[dof] = out;
}

// The FP32 stencil kernels on small levels: four threads per (node, row), one
// part of the row each (stencil_part), combined in shared memory in the order
// stencil_row uses, so both kernels give the same bits.  384 threads: 32
// consecutive nodes x 3 rows x 4 parts.  The update's vector reads are issued
// before the row's, so they overlap.
constexpr int kSplitThreads = 384;
constexpr int64_t kSplitMaxNodes = 16384;

template <int MODE>
__global__ void __launch_bounds__(kSplitThreads) k_stencil_split(
    MgDims d, const float* __restrict__ A, const uint8_t* __restrict__ act,
    const float* __restrict__ x, const float* __restrict__ b, const float* __restrict__ invdiag,
    float omega, float* __restrict__ y, ChebStep ch) {
  __shared__ float parts[3][3][32];
  const int t = threadIdx.x, q = t / 96, r = (t / 32) % 3, lane = t & 31;
  const int64_t n = int64_t(blockIdx.x) * 32 + lane;
  const bool valid = n < int64_t(d.nnx) * d.nny * d.nnz;
  const int64_t dof = 3 * n + r;
  float* dir = static_cast<float*>(ch.dir_);
  bool ac = false;
  float xv = 0.0f, bv = 0.0f, dv = 0.0f, dprev = 0.0f;
  if (q == 0 && valid) {
    ac = act[dof] != 0;
    if (MODE == kSmooth || MODE == kCheb) xv = x[dof];
    if (MODE != kApply) bv = b[dof];
    if (MODE == kSmooth || MODE == kCheb) dv = invdiag[dof];
    if (MODE == kCheb && ch.step > 0) dprev = dir[dof];
  }
  float p = 0.0f;
  if (valid) {
    int a, bb, c;
    node_abc(d, n, a, bb, c);
    p = stencil_part<float, false>(d, A, x, a, bb, c, r, q);
  }
  if (q > 0) parts[q - 1][r][lane] = p;
  __syncthreads();
  if (q != 0 || !valid) return;
  const float s = ((p + parts[0][r][lane]) + parts[1][r][lane]) + parts[2][r][lane];
  float dnew;
  const float out = stencil_update<float, MODE>(ac, s, xv, bv, dv, omega, ch.coef, ch.step,
                                                ac ? dprev : 0.0f, dnew);
  if (MODE == kCheb) dir[dof] = dnew;
  y[dof] = out;
}

// Power iteration for lambda_max(D^-1 A) of one stencil level: v on the
// active DOFs from a fixed hash, then w = D^-1 A v, v = w / |w|; |w| -> lam.
template <class T>
__global__ void k_pi_init(const uint8_t* __restrict__ act, int64_t n, T* __restrict__ v) {
  for (int64_t i = blockIdx.x * int64_t(kThreads) + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * kThreads) {
    uint32_t h = uint32_t(i) * 2654435761u;
    h ^= h >> 16;
    v[i] = act[i] ? T(0.5) + T(h & 0xffff) * T(1.0 / 65536.0) : T(0);
  }
}
template <class T>
__global__ void k_pi_dinv(T* __restrict__ w, const T* __restrict__ invdiag, int64_t n) {
  for (int64_t i = blockIdx.x * int64_t(kThreads) + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * kThreads)
    w[i] *= invdiag[i];
}
template <class T>
__global__ void k_pi_scale(T* __restrict__ v, const T* __restrict__ w,
                           const double* __restrict__ nrm2, int64_t n) {
  const double q = nrm2[0] > 0.0 ? 1.0 / sqrt(nrm2[0]) : 0.0;
  for (int64_t i = blockIdx.x * int64_t(kThreads) + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * kThreads)
    v[i] = T(q) * w[i];
}
__global__ void k_pi_lambda(const double* __restrict__ nrm2, double safety,
                            double* __restrict__ lam) {
  if (threadIdx.x == 0) lam[0] = safety * sqrt(nrm2[0] > 0.0 ? nrm2[0] : 1.0);
}

// Chebyshev coefficients on [lmax / ratio, lmax]: theta, delta the interval's
// centre and half-width, rho_0 = delta / theta, rho_k = 1 / (2 theta / delta -
// rho_{k-1}); thread k writes step k's pair.
__global__ void k_cheb_table(const double* __restrict__ lam, double ratio, int m,
                             float* __restrict__ coef) {
  const int k = threadIdx.x;
  if (k >= m) return;
  const double lmax = lam[0], lmin = lmax / ratio;
  const double theta = 0.5 * (lmax + lmin), delta = 0.5 * (lmax - lmin), sig = theta / delta;
  double rp = 1.0 / sig, rk = rp;
  for (int i = 1; i <= k; ++i) {
    rp = rk;
    rk = 1.0 / (2.0 * sig - rp);
  }
  if (k == 0) {
    coef[0] = float(1.0 / theta);
    coef[1] = 0.0f;
  } else {
    coef[2 * k] = float(rk * rp);
    coef[2 * k + 1] = float(2.0 * rk / delta);
  }
}

// x = omega * invdiag .* b (the first smoother sweep from a zero iterate).
template <class T>
__global__ void k_jacobi_first(const T* __restrict__ b, const T* __restrict__ invdiag, T omega,
                               int64_t n, T* __restrict__ x) {
  for (int64_t i = blockIdx.x * int64_t(kThreads) + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * kThreads)
    x[i] = omega * invdiag[i] * b[i];
}

// Boundary-aligned coarsening (MgDims::align): on an odd fine axis the last
// fine node (index Ef) is the coincident node of coarse node (Ef + 1) / 2.
__device__ __forceinline__ bool tail_node(int i, int Ef, int align) {
  return align && (Ef & 1) && i == Ef;
}
// Weight of fine node i (= 2N + d) in coarse node N along one axis.
template <class T>
__device__ __forceinline__ T axis_w(int i, int N, int d, int Ef, int align) {
  if (tail_node(i, Ef, align)) return N == (Ef + 1) / 2 ? T(1) : T(0);
  return d == 0 ? T(1) : T(0.5);
}

// Restriction R = P^T: coarse node N gathers the (up to 27) fine nodes
// 2N + delta, delta in {-1,0,1}^3, weight prod(1 or 1/2).  Inactive coarse DOFs
// get 0; fine residuals are already 0 on inactive fine DOFs.  One thread per
// coarse node on a 3D grid (x fastest), 32-bit index arithmetic.
// The restricted residual at coarse node (a, b, c): s[k] = sum of the (up to 27)
// fine nodes' component k times their weights, in a fixed order.
template <class T, bool COH>
__device__ __forceinline__ void restrict_node(const MgDims& fd, const MgDims& cd, const T* rf,
                                              int a, int b, int c, T (&s)[3]) {
  s[0] = s[1] = s[2] = T(0);
#pragma unroll
  for (int dz = -1; dz <= 1; ++dz) {
    const int k = 2 * c + dz;
    if (k < 0 || k >= fd.nnz) continue;
    const T wz = axis_w<T>(k, c, dz, fd.ez, cd.align);
#pragma unroll
    for (int dy = -1; dy <= 1; ++dy) {
      const int j = 2 * b + dy;
      if (j < 0 || j >= fd.nny) continue;
      const T wy = axis_w<T>(j, b, dy, fd.ey, cd.align) * wz;
#pragma unroll
      for (int dx = -1; dx <= 1; ++dx) {
        const int i = 2 * a + dx;
        if (i < 0 || i >= fd.nnx) continue;
        const T w = axis_w<T>(i, a, dx, fd.ex, cd.align) * wy;
        const T* q = rf + 3 * ((int64_t(k) * fd.nny + j) * fd.nnx + i);
        s[0] += w * vload<T, COH>(q);
        s[1] += w * vload<T, COH>(q + 1);
        s[2] += w * vload<T, COH>(q + 2);
      }
    }
  }
}

template <class T>
__global__ void __launch_bounds__(256) k_restrict(MgDims fd, MgDims cd, const T* __restrict__ rf,
                                                  const uint8_t* __restrict__ cact,
                                                  T* __restrict__ bc, FirstStep<T> first) {
  const int a = blockIdx.x * 32 + threadIdx.x, b = blockIdx.y * 8 + threadIdx.y, c = blockIdx.z;
  if (a >= cd.nnx || b >= cd.nny) return;
  T s[3];
  restrict_node<T, false>(fd, cd, rf, a, b, c, s);
  const int64_t n = (int64_t(c) * cd.nny + b) * cd.nnx + a;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const int64_t dof = 3 * n + k;
    const bool ac = cact[dof] != 0;
    const T bv = ac ? s[k] : T(0);
    bc[dof] = bv;
    if (first.kind == 1) {
      first.x[dof] = first.omega * first.dinv[dof] * bv;
    } else if (first.kind == 2) {
      T dnew;
      first.x[dof] = stencil_update<T, kCheb>(ac, T(0), T(0), bv, first.dinv[dof], T(0),
                                              first.coef, 0, T(0), dnew);
      first.chd[dof] = dnew;
    }
  }
}

// The prolonged correction at fine node (a, b, c): per axis one coarse node
// (an even fine node, or the aligned tail node) or two at weight 1/2.
template <class T, bool COH>
__device__ __forceinline__ void prolong_node(const MgDims& fd, const MgDims& cd, const T* ec,
                                             int a, int b, int c, T (&s)[3]) {
  const bool ta = tail_node(a, fd.ex, cd.align), tb = tail_node(b, fd.ey, cd.align),
             tc = tail_node(c, fd.ez, cd.align);
  const int na = (a & 1) && !ta ? 2 : 1, nb = (b & 1) && !tb ? 2 : 1, ncz = (c & 1) && !tc ? 2 : 1;
  const int ia0 = ta ? (a + 1) >> 1 : a >> 1, ia1 = (a + 1) >> 1;
  const int ib0 = tb ? (b + 1) >> 1 : b >> 1, ib1 = (b + 1) >> 1;
  const int ic0 = tc ? (c + 1) >> 1 : c >> 1, ic1 = (c + 1) >> 1;
  const T w = (na == 2 ? T(0.5) : T(1)) * (nb == 2 ? T(0.5) : T(1)) * (ncz == 2 ? T(0.5) : T(1));
  s[0] = s[1] = s[2] = T(0);
#pragma unroll
  for (int zz = 0; zz < 2; ++zz) {
    if (zz >= ncz) continue;
    const int k = zz ? ic1 : ic0;
#pragma unroll
    for (int yy = 0; yy < 2; ++yy) {
      if (yy >= nb) continue;
      const int j = yy ? ib1 : ib0;
#pragma unroll
      for (int xx = 0; xx < 2; ++xx) {
        if (xx >= na) continue;
        const int i = xx ? ia1 : ia0;
        if (i >= cd.nnx || j >= cd.nny || k >= cd.nnz) continue;
        const T* q = ec + 3 * ((int64_t(k) * cd.nny + j) * cd.nnx + i);
        s[0] += w * vload<T, COH>(q);
        s[1] += w * vload<T, COH>(q + 1);
        s[2] += w * vload<T, COH>(q + 2);
      }
    }
  }
}

// Prolongation + correction: x_f += P e_c on active fine DOFs.  One thread per
// fine node on a 3D grid.
template <class T>
__global__ void __launch_bounds__(256) k_prolong_add(MgDims fd, MgDims cd,
                                                     const T* __restrict__ ec,
                                                     const uint8_t* __restrict__ fact,
                                                     T* __restrict__ xf) {
  const int a = blockIdx.x * 32 + threadIdx.x, b = blockIdx.y * 8 + threadIdx.y, c = blockIdx.z;
  if (a >= fd.nnx || b >= fd.nny) return;
  const int64_t n = (int64_t(c) * fd.nny + b) * fd.nnx + a;
  // The iterate and the mask are read unconditionally, in parallel with the
  // coarse values: a read under the mask's branch would wait for the mask first.
  const T x0 = xf[3 * n], x1 = xf[3 * n + 1], x2 = xf[3 * n + 2];
  const bool f0 = fact[3 * n] != 0, f1 = fact[3 * n + 1] != 0, f2 = fact[3 * n + 2] != 0;
  T s[3];
  prolong_node<T, false>(fd, cd, ec, a, b, c, s);
  if (f0) xf[3 * n] = x0 + s[0];
  if (f1) xf[3 * n + 1] = x1 + s[1];
  if (f2) xf[3 * n + 2] = x2 + s[2];
}

// ---------------------------------------------------------- coarsest solve
// Dense A (row-major, nc x nc) from the coarsest stencil over the compact
// numbering cidx (-1 = inactive): node n writes its self block and, for every
// forward block, the entry and its transpose -- each entry exactly once.
template <class T>
__global__ void k_dense_from_stencil(MgDims d, const T* __restrict__ A,
                                     const int* __restrict__ cidx, int nc,
                                     double* __restrict__ D) {
  const int64_t nn = int64_t(d.nnx) * d.nny * d.nnz;
  for (int64_t n = blockIdx.x * int64_t(kThreads) + threadIdx.x; n < nn;
       n += int64_t(gridDim.x) * kThreads) {
    int a, b, c;
    node_abc(d, n, a, b, c);
    for (int j = 0; j < 14; ++j) {
      const int di = 13 + j;
      const int i = a + di % 3 - 1, jj = b + (di / 3) % 3 - 1, k = c + di / 9 - 1;
      if (i < 0 || i >= d.nnx || jj < 0 || jj >= d.nny || k >= d.nnz) continue;
      const int64_t m = (int64_t(k) * d.nny + jj) * d.nnx + i;
      for (int c1 = 0; c1 < 3; ++c1) {
        const int row = cidx[3 * n + c1];
        if (row < 0) continue;
        for (int c2 = 0; c2 < 3; ++c2) {
          const int col = cidx[3 * m + c2];
          if (col < 0) continue;
          const double v = double(A[int64_t(j * 9 + c1 * 3 + c2) * nn + n]);
          D[int64_t(row) * nc + col] = v;
          if (j > 0) D[int64_t(col) * nc + row] = v;
        }
      }
    }
  }
}

// Blocked right-looking Cholesky, panel width 32.  Step 1: factor the diagonal
// block in shared memory (one CTA); a non-positive pivot sets *fail.
__global__ void k_chol_diag(double* __restrict__ D, int nc, int k0, int* __restrict__ fail) {
  __shared__ double s[32][33];
  const int nb = min(32, nc - k0);
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 32 threads
  if (tx < nb && ty < nb) s[ty][tx] = D[int64_t(k0 + ty) * nc + k0 + tx];
  __syncthreads();
  for (int j = 0; j < nb; ++j) {
    if (tx == 0 && ty == 0) {
      const double p = s[j][j];
      if (!(p > 0.0)) *fail = 1;
      s[j][j] = p > 0.0 ? sqrt(p) : 1.0;
    }
    __syncthreads();
    if (ty == 0 && tx > j && tx < nb) s[tx][j] /= s[j][j];
    __syncthreads();
    if (ty > j && tx > j && ty < nb && tx <= ty) s[ty][tx] -= s[ty][j] * s[tx][j];
    __syncthreads();
  }
  if (tx < nb && ty < nb && tx <= ty) D[int64_t(k0 + ty) * nc + k0 + tx] = s[ty][tx];
}

// Step 2: rows below the diagonal block: L[i, k0:k0+nb] = A[i, .] L_kk^-T.
__global__ void k_chol_panel(double* __restrict__ D, int nc, int k0) {
  __shared__ double L[32][33];
  const int nb = min(32, nc - k0);
  for (int t = threadIdx.x; t < 32 * 32; t += blockDim.x) {
    const int r = t / 32, c = t % 32;
    L[r][c] = (r < nb && c < nb && c <= r) ? D[int64_t(k0 + r) * nc + k0 + c] : 0.0;
  }
  __syncthreads();
  const int i = k0 + nb + blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nc) return;
  double row[32];
  for (int c = 0; c < nb; ++c) row[c] = D[int64_t(i) * nc + k0 + c];
  for (int c = 0; c < nb; ++c) {
    double v = row[c];
    for (int t = 0; t < c; ++t) v -= row[t] * L[c][t];
    row[c] = v / L[c][c];
  }
  for (int c = 0; c < nb; ++c) D[int64_t(i) * nc + k0 + c] = row[c];
}

// Step 3: trailing update of the lower triangle, 32x32 tiles.
__global__ void k_chol_update(double* __restrict__ D, int nc, int k0) {
  const int nb = min(32, nc - k0);
  const int r0 = k0 + nb + blockIdx.y * 32, c0 = k0 + nb + blockIdx.x * 32;
  if (c0 > r0 + 31) return;
  __shared__ double Li[32][33], Lj[32][33];
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  for (int yy = ty; yy < 32; yy += blockDim.x / 32) {
    Li[yy][tx] = (r0 + yy < nc && tx < nb) ? D[int64_t(r0 + yy) * nc + k0 + tx] : 0.0;
    Lj[yy][tx] = (c0 + yy < nc && tx < nb) ? D[int64_t(c0 + yy) * nc + k0 + tx] : 0.0;
  }
  __syncthreads();
  for (int yy = ty; yy < 32; yy += blockDim.x / 32) {
    const int i = r0 + yy, j = c0 + tx;
    if (i >= nc || j >= nc || j > i) continue;
    double s = 0.0;
    for (int t = 0; t < nb; ++t) s += Li[yy][t] * Lj[tx][t];
    D[int64_t(i) * nc + j] -= s;
  }
}

// Explicit inverse of the coarsest operator from its Cholesky factor, for small
// coarsest levels: thread j forms column j of L^-1 by forward substitution, then
// Ainv = L^-T L^-1 (both FP64).  Each V-cycle then needs one dense matvec.
// Column j of L^-1 by forward substitution, one warp per column: the inner
// product of row i of L with the column's entries above i is split over the
// lanes and reduced by shuffles, so a column costs nc short steps instead of a
// serial O(nc^2) chain (the factor and the column stay in L2).
__global__ void k_chol_invert_L(const double* __restrict__ L, int nc, double* __restrict__ Li) {
  const int j = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (j >= nc) return;  // warp-uniform
  for (int i = lane; i < j; i += 32) Li[int64_t(i) * nc + j] = 0.0;
  for (int i = j; i < nc; ++i) {
    double part = 0.0;
    for (int k = j + lane; k < i; k += 32) part += L[int64_t(i) * nc + k] * Li[int64_t(k) * nc + j];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
    if (lane == 0) Li[int64_t(i) * nc + j] = ((i == j ? 1.0 : 0.0) - part) / L[int64_t(i) * nc + i];
    __syncwarp();  // the new entry is read by every lane from the next row on
  }
}

__global__ void k_chol_inverse(const double* __restrict__ Li, int nc, double* __restrict__ Ainv) {
  const int i = blockIdx.y * 16 + threadIdx.y, j = blockIdx.x * 16 + threadIdx.x;
  if (i >= nc || j >= nc) return;
  double s = 0.0;
  for (int k = max(i, j); k < nc; ++k) s += Li[int64_t(k) * nc + i] * Li[int64_t(k) * nc + j];
  Ainv[int64_t(i) * nc + j] = s;
}

// x = Ainv b on the compact numbering, gathered from / scattered to the level
// vector; one warp per row of Ainv.
template <class T>
__global__ void k_coarse_inv_apply(const double* __restrict__ Ainv, int nc,
                                   const int* __restrict__ cidx, const int* __restrict__ cdof,
                                   int64_t ndof, const T* __restrict__ b, T* __restrict__ x) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int64_t dd = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; dd < ndof;
       dd += int64_t(gridDim.x) * blockDim.x)
    if (cidx[dd] < 0) x[dd] = T(0);
  for (int r = warp; r < nc; r += nwarps) {
    double s = 0.0;
    for (int k = lane; k < nc; k += 32) s += Ainv[int64_t(r) * nc + k] * double(b[cdof[k]]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) x[cdof[r]] = T(s);
  }
}

// Forward and backward substitution with the factor, one CTA; the coarsest
// right-hand side is gathered from / scattered to the stencil-level vector.
template <class T>
__global__ void k_chol_solve(const double* __restrict__ L, int nc, const int* __restrict__ cidx,
                             int64_t ndof, const T* __restrict__ b, T* __restrict__ x,
                             double* __restrict__ work) {
  for (int64_t d = threadIdx.x; d < ndof; d += blockDim.x) {
    const int ci = cidx[d];
    if (ci >= 0) work[ci] = double(b[d]);
  }
  __syncthreads();
  for (int j = 0; j < nc; ++j) {  // L y = b
    __shared__ double yj;
    if (threadIdx.x == 0) {
      yj = work[j] / L[int64_t(j) * nc + j];
      work[j] = yj;
    }
    __syncthreads();
    for (int i = j + 1 + threadIdx.x; i < nc; i += blockDim.x) work[i] -= L[int64_t(i) * nc + j] * yj;
    __syncthreads();
  }
  for (int j = nc - 1; j >= 0; --j) {  // L^T x = y
    __shared__ double xj;
    if (threadIdx.x == 0) {
      xj = work[j] / L[int64_t(j) * nc + j];
      work[j] = xj;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < j; i += blockDim.x) work[i] -= L[int64_t(j) * nc + i] * xj;
    __syncthreads();
  }
  for (int64_t d = threadIdx.x; d < ndof; d += blockDim.x) {
    const int ci = cidx[d];
    x[d] = ci >= 0 ? T(work[ci]) : T(0);
  }
}
}  // namespace

// Level 1's Galerkin matrices of the coarse elements on the fast path
// (spos[ce] < 0: no aligned half element, every coarse DOF active, every fine
// DOF of every existing child kept), where the matrix is sum_c f_c G_c.  The
// sum runs over the children inside the grid with a nonzero modulus, in child
// order, one fused multiply-add per term -- k_galerkin's arithmetic, so the
// entries are bit-identical.  A block of 576 threads, one per matrix entry,
// holds its entry of the 8 G_c in registers and walks a batch of elements: the
// 576 entries of an element are 576 consecutive floats written by consecutive
// threads.
constexpr int kGalFastBatch = 32;  // elements per block step
__global__ void __launch_bounds__(576) k_galerkin1_fast(MgDims fd, MgDims cd,
                                                        const float* __restrict__ ef,
                                                        const int* __restrict__ spos,
                                                        const float* __restrict__ G,
                                                        float* __restrict__ Kc) {
  __shared__ float sf[kGalFastBatch][8];
  __shared__ int sfast[kGalFastBatch];
  const int rc = threadIdx.x;  // this thread's matrix entry, 0 .. 575
  float g[8];                  // its 8 child blocks' entries, for every element
#pragma unroll
  for (int ch = 0; ch < 8; ++ch) g[ch] = G[ch * 576 + rc];
  const int64_t nce = int64_t(cd.ex) * cd.ey * cd.ez;
  for (int64_t base = int64_t(blockIdx.x) * kGalFastBatch; base < nce;
       base += int64_t(gridDim.x) * kGalFastBatch) {
    __syncthreads();  // the previous step's sf / sfast consumed
    if (threadIdx.x < kGalFastBatch * 8) {
      const int el = threadIdx.x >> 3, ch = threadIdx.x & 7;
      const int64_t ce = base + el;
      float f = 0.0f;
      if (ce < nce) {
        const int I = int(ce % cd.ex), J = int((ce / cd.ex) % cd.ey),
                  K = int(ce / (int64_t(cd.ex) * cd.ey));
        const int fi = 2 * I + cx(ch), fj = 2 * J + cy(ch), fk = 2 * K + cz(ch);
        if (fi < fd.ex && fj < fd.ey && fk < fd.ez) f = ef[(int64_t(fk) * fd.ey + fj) * fd.ex + fi];
      }
      sf[el][ch] = f;
      if (ch == 0) sfast[el] = ce < nce && spos[ce] < 0;
    }
    __syncthreads();
    for (int el = 0; el < kGalFastBatch; ++el) {
      if (!sfast[el]) continue;  // uniform over the block
      float acc = 0.0f;
#pragma unroll
      for (int ch = 0; ch < 8; ++ch) {
        const float f = sf[el][ch];
        if (f != 0.0f) acc = __fmaf_rn(f, g[ch], acc);
      }
      Kc[(base + el) * 576 + rc] = acc;
    }
  }
}

template <class T>
void mg_galerkin_level1(const MgDims& fd, const MgDims& cd, const T* ef, const uint8_t* fact,
                        const uint8_t* cact, const T* Ke, const T* G, T* Kc, cudaStream_t s,
                        const int* spos) {
  const int64_t nce = int64_t(cd.ex) * cd.ey * cd.ez;
  const int* skip = nullptr;
  if constexpr (sizeof(T) == 4) {
    if (spos != nullptr) {
      const int64_t steps = (nce + kGalFastBatch - 1) / kGalFastBatch;
      const int nb = int(std::min<int64_t>(steps, 152 * 6));
      k_galerkin1_fast<<<nb, 576, 0, s>>>(fd, cd, ef, spos, G, Kc);
      TG_LAUNCH_CHECK();
      skip = spos;
    }
  }
  k_galerkin<T, true><<<nblk(nce, 4), 128, 0, s>>>(fd, cd, ef, fact, cact, Ke, G, nullptr, Kc,
                                                   skip);
  TG_LAUNCH_CHECK();
}

template <class T>
void mg_galerkin_coarse(const MgDims& fd, const MgDims& cd, const T* Kf, const uint8_t* cact,
                        T* Kc, cudaStream_t s) {
  const int64_t nce = int64_t(cd.ex) * cd.ey * cd.ez;
  k_galerkin<T, false><<<nblk(nce, 4), 128, 0, s>>>(fd, cd, nullptr, nullptr, cact, nullptr,
                                                    nullptr, Kf, Kc, nullptr);
  TG_LAUNCH_CHECK();
}

template <class T>
void mg_assemble_stencil(const MgDims& d, const T* Kel, const uint8_t* act, T* A, T* invdiag,
                         cudaStream_t s) {
  const int64_t nn = int64_t(d.nnx) * d.nny * d.nnz;
  k_assemble_stencil<T><<<nblk(nn), kThreads, 0, s>>>(d, Kel, act, A, invdiag);
  TG_LAUNCH_CHECK();
}

void mg_to_float(const double* src, float* dst, int64_t n, cudaStream_t s) {
  k_to_float<float><<<nblk(n), kThreads, 0, s>>>(src, dst, n);
  TG_LAUNCH_CHECK();
}

template <class T>
void mg_stencil_op(int mode, const MgDims& d, const T* A, const uint8_t* act, const T* x,
                   const T* b, const T* invdiag, T omega, T* y, cudaStream_t s,
                   ChebStep ch) {
  const int64_t nn = int64_t(d.nnx) * d.nny * d.nnz;
  if constexpr (sizeof(T) == 4) {
    if (nn <= kSplitMaxNodes) {
      const unsigned ns = unsigned((nn + 31) / 32);
      if (mode == kApply)
        k_stencil_split<kApply><<<ns, kSplitThreads, 0, s>>>(d, A, act, x, b, invdiag, omega, y, ch);
      else if (mode == kResidual)
        k_stencil_split<kResidual><<<ns, kSplitThreads, 0, s>>>(d, A, act, x, b, invdiag, omega, y,
                                                                ch);
      else if (mode == kCheb)
        k_stencil_split<kCheb><<<ns, kSplitThreads, 0, s>>>(d, A, act, x, b, invdiag, omega, y, ch);
      else
        k_stencil_split<kSmooth><<<ns, kSplitThreads, 0, s>>>(d, A, act, x, b, invdiag, omega, y,
                                                              ch);
      TG_LAUNCH_CHECK();
      return;
    }
  }
  const int64_t items = (nn + 31) / 32 * 96;
  const unsigned nb = unsigned((items + kStencilThreads - 1) / kStencilThreads);
  const unsigned nt = kStencilThreads;
  if (mode == kApply)
    k_stencil_op<T, kApply><<<nb, nt, 0, s>>>(d, A, act, x, b, invdiag, omega, y, ch);
  else if (mode == kResidual)
    k_stencil_op<T, kResidual><<<nb, nt, 0, s>>>(d, A, act, x, b, invdiag, omega, y, ch);
  else if (mode == kCheb)
    k_stencil_op<T, kCheb><<<nb, nt, 0, s>>>(d, A, act, x, b, invdiag, omega, y, ch);
  else
    k_stencil_op<T, kSmooth><<<nb, nt, 0, s>>>(d, A, act, x, b, invdiag, omega, y, ch);
  TG_LAUNCH_CHECK();
}

void mg_cheb_table(const double* lam, double ratio, int m, float* coef, cudaStream_t s) {
  if (m < 1 || 2 * m > kChebCoefStride) raise(TG_EINVAL, "Chebyshev degree out of range");
  k_cheb_table<<<1, 32, 0, s>>>(lam, ratio, m, coef);
  TG_LAUNCH_CHECK();
}

template <class T>
void mg_lambda_max(const MgDims& d, const T* A, const uint8_t* act, const T* invdiag, T* v,
                   T* w, int iters, double safety, double* part, double* nrm2, double* lam,
                   cudaStream_t s) {
  const int64_t n = 3 * int64_t(d.nnx) * d.nny * d.nnz;
  const int nbk = nblk(n);
  k_pi_init<T><<<nbk, kThreads, 0, s>>>(act, n, v);
  TG_LAUNCH_CHECK();
  for (int it = 0; it < iters; ++it) {
    mg_stencil_op<T>(kApply, d, A, act, v, nullptr, nullptr, T(0), w, s);
    k_pi_dinv<T><<<nbk, kThreads, 0, s>>>(w, invdiag, n);
    TG_LAUNCH_CHECK();
    if constexpr (sizeof(T) == 4)
      launch_dot_f(w, w, n, part, nrm2, s);
    else
      launch_dot(w, w, n, part, nrm2, s);
    k_pi_scale<T><<<nbk, kThreads, 0, s>>>(v, w, nrm2, n);
    TG_LAUNCH_CHECK();
  }
  k_pi_lambda<<<1, 32, 0, s>>>(nrm2, safety, lam);
  TG_LAUNCH_CHECK();
}
template void mg_lambda_max<float>(const MgDims&, const float*, const uint8_t*, const float*,
                                   float*, float*, int, double, double*, double*, double*,
                                   cudaStream_t);

template <class T>
void mg_jacobi_first(const T* b, const T* invdiag, T omega, int64_t n, T* x, cudaStream_t s) {
  k_jacobi_first<T><<<nblk(n), kThreads, 0, s>>>(b, invdiag, omega, n, x);
  TG_LAUNCH_CHECK();
}

template <class T>
void mg_restrict(const MgDims& fd, const MgDims& cd, const T* rf, const uint8_t* cact, T* bc,
                 cudaStream_t s, FirstStep<T> first) {
  const dim3 grid((cd.nnx + 31) / 32, (cd.nny + 7) / 8, cd.nnz);
  k_restrict<T><<<grid, dim3(32, 8), 0, s>>>(fd, cd, rf, cact, bc, first);
  TG_LAUNCH_CHECK();
}

template <class T>
void mg_prolong_add(const MgDims& fd, const MgDims& cd, const T* ec, const uint8_t* fact, T* xf,
                    cudaStream_t s) {
  const dim3 grid((fd.nnx + 31) / 32, (fd.nny + 7) / 8, fd.nnz);
  k_prolong_add<T><<<grid, dim3(32, 8), 0, s>>>(fd, cd, ec, fact, xf);
  TG_LAUNCH_CHECK();
}

template <class T>
void mg_dense_from_stencil(const MgDims& d, const T* A, const int* cidx, int nc, double* D,
                           cudaStream_t s) {
  const int64_t nn = int64_t(d.nnx) * d.nny * d.nnz;
  TG_CUDA(cudaMemsetAsync(D, 0, sizeof(double) * size_t(nc) * nc, s));
  k_dense_from_stencil<T><<<nblk(nn), kThreads, 0, s>>>(d, A, cidx, nc, D);
  TG_LAUNCH_CHECK();
}

void mg_cholesky(double* D, int nc, int* fail, cudaStream_t s) {
  for (int k0 = 0; k0 < nc; k0 += 32) {
    k_chol_diag<<<1, 1024, 0, s>>>(D, nc, k0, fail);
    TG_LAUNCH_CHECK();
    const int rest = nc - k0 - 32;
    if (rest <= 0) break;
    k_chol_panel<<<(rest + 127) / 128, 128, 0, s>>>(D, nc, k0);
    TG_LAUNCH_CHECK();
    const int tiles = (rest + 31) / 32;
    k_chol_update<<<dim3(tiles, tiles), 256, 0, s>>>(D, nc, k0);
    TG_LAUNCH_CHECK();
  }
}

void mg_chol_inverse(const double* L, int nc, double* Li, double* Ainv, cudaStream_t s) {
  k_chol_invert_L<<<(nc + 3) / 4, 128, 0, s>>>(L, nc, Li);  // a warp per column
  TG_LAUNCH_CHECK();
  const dim3 grid((nc + 15) / 16, (nc + 15) / 16);
  k_chol_inverse<<<grid, dim3(16, 16), 0, s>>>(Li, nc, Ainv);
  TG_LAUNCH_CHECK();
}

template <class T>
void mg_coarse_inv_apply(const double* Ainv, int nc, const int* cidx, const int* cdof,
                         int64_t ndof, const T* b, T* x, cudaStream_t s) {
  k_coarse_inv_apply<T><<<std::max(1, std::min(152, (nc + 7) / 8)), 256, 0, s>>>(Ainv, nc, cidx, cdof, ndof, b, x);
  TG_LAUNCH_CHECK();
}

template <class T>
void mg_chol_solve(const double* L, int nc, const int* cidx, int64_t ndof, const T* b, T* x,
                   double* work, cudaStream_t s) {
  k_chol_solve<T><<<1, 512, 0, s>>>(L, nc, cidx, ndof, b, x, work);
  TG_LAUNCH_CHECK();
}

#define TG_INST(T)                                                                            \
  template void mg_stencil_op<T>(int, const MgDims&, const T*, const uint8_t*, const T*,      \
                                 const T*, const T*, T, T*, cudaStream_t, ChebStep);          \
  template void mg_jacobi_first<T>(const T*, const T*, T, int64_t, T*, cudaStream_t);         \
  template void mg_restrict<T>(const MgDims&, const MgDims&, const T*, const uint8_t*, T*,    \
                               cudaStream_t, FirstStep<T>);                                   \
  template void mg_prolong_add<T>(const MgDims&, const MgDims&, const T*, const uint8_t*, T*, \
                                  cudaStream_t);                                              \
  template void mg_chol_solve<T>(const double*, int, const int*, int64_t, const T*, T*,       \
                                 double*, cudaStream_t);                                      \
  template void mg_coarse_inv_apply<T>(const double*, int, const int*, const int*, int64_t,    \
                                       const T*, T*, cudaStream_t);                           \
  template void mg_galerkin_level1<T>(const MgDims&, const MgDims&, const T*, const uint8_t*,  \
                                      const uint8_t*, const T*, const T*, T*, cudaStream_t,   \
                                      const int*);                                            \
  template void mg_galerkin_coarse<T>(const MgDims&, const MgDims&, const T*, const uint8_t*,  \
                                      T*, cudaStream_t);                                      \
  template void mg_assemble_stencil<T>(const MgDims&, const T*, const uint8_t*, T*, T*,       \
                                       cudaStream_t);                                         \
  template void mg_dense_from_stencil<T>(const MgDims&, const T*, const int*, int, double*,   \
                                         cudaStream_t);
TG_INST(double)
TG_INST(float)
#undef TG_INST



// ------------------------------------------------- fused coarse V-cycle
// The small levels of the FP32 V-cycle -- from the first level with at most
// kFusedMaxNodes nodes down to the coarsest -- in one launch of one thread-block
// cluster (off by default: a launch per step, 3-4 us each with the four-thread
// stencil kernel, measured faster than a phase of this kernel, ~9 us on 16
// SMs).  Launch by launch, each step on these levels is a kernel of a few
// thousand DOFs whose cost is its latency.  Here every step of the same
// V-cycle is a phase of one kernel -- a
// cluster-stride loop with the arithmetic and summation order of the separate
// kernels (stencil_row, restrict_node, prolong_node, the coarsest inverse) --
// and phases are separated by the cluster's hardware barrier (release/acquire
// at cluster scope, no spin loop).  The restriction into a level and that
// level's first smoothing step (from a zero iterate, so it needs no operator)
// share a phase.  Vectors written in earlier phases are read through L2
// (another SM of the cluster may have written them).  The iterate ping-pongs
// between each level's two buffers exactly as the launch-by-launch V-cycle does.
namespace {

// Every thread of the cluster arrives; writes before the barrier (global and
// shared memory) are visible to every thread of the cluster after it.
__device__ __forceinline__ void cluster_sync_all() {
  asm volatile(
      "barrier.cluster.arrive.release.aligned;\n\t"
      "barrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// Work items of a per-DOF phase: chunks of 32 nodes x 3 components, one
// component per warp, so a warp's stencil reads are coalesced.
__device__ __forceinline__ void dof_item(int64_t it, const MgDims& d, int& a, int& b, int& c,
                                         int& r, int64_t& n) {
  const int64_t chunk = it / 96;
  r = int((it / 32) % 3);
  n = chunk * 32 + (it & 31);
  node_abc(d, n, a, b, c);
}

__global__ void __launch_bounds__(kFusedThreads, 1) k_coarse_vcycle(FusedCoarse fc) {
  const int64_t tid = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  const int64_t nthreads = int64_t(gridDim.x) * blockDim.x;
  const int top = fc.nlev - 1;  // the coarsest
  int cur[kFusedMaxLevels] = {};  // 0: the iterate is in xp, 1: in xq
  auto X = [&](int i) { return cur[i] ? fc.L[i].xq : fc.L[i].xp; };
  auto O = [&](int i) { return cur[i] ? fc.L[i].xp : fc.L[i].xq; };
  auto nitems = [&](int i) { return ((int64_t(fc.L[i].d.nnx) * fc.L[i].d.nny * fc.L[i].d.nnz + 31) / 32) * 96; };

  // One smoothing step of level i from its current iterate (or from zero) into
  // the other buffer: Chebyshev step k, or damped Jacobi (whose first sweep from
  // zero writes the iterate's own buffer, as the separate launches do).
  auto smooth = [&](int i, int k, bool from_zero) {
    const FusedLevel& L = fc.L[i];
    const float* xin = X(i);
    const bool in_place = from_zero && fc.cheb_m == 0;
    float* xout = in_place ? X(i) : O(i);
    const int64_t ni = nitems(i), nn = int64_t(L.d.nnx) * L.d.nny * L.d.nnz;
    for (int64_t it = tid; it < ni; it += nthreads) {
      int a, b, c, r;
      int64_t n;
      dof_item(it, L.d, a, b, c, r, n);
      if (n >= nn) continue;
      const int64_t dof = 3 * n + r;
      const float s = from_zero ? 0.0f : stencil_row<float, true>(L.d, L.A, xin, a, b, c, r);
      const float xv = from_zero ? 0.0f : __ldcg(xin + dof);
      const bool ac = L.act[dof] != 0;
      float out, dnew;
      if (fc.cheb_m > 0) {
        out = stencil_update<float, kCheb>(ac, s, xv, __ldcg(L.b + dof), L.dinv[dof], 0.0f, L.coef,
                                           k, (k > 0 && ac) ? __ldcg(L.chd + dof) : 0.0f, dnew);
        L.chd[dof] = dnew;
      } else {
        out = stencil_update<float, kSmooth>(ac, s, xv, __ldcg(L.b + dof), L.dinv[dof], fc.omega,
                                             nullptr, 0, 0.0f, dnew);
      }
      xout[dof] = out;
    }
    if (!in_place) cur[i] ^= 1;
  };
  // r = b - A x of level i into its other buffer (the iterate stays).
  auto residual = [&](int i) {
    const FusedLevel& L = fc.L[i];
    const float* xin = X(i);
    float* rout = O(i);
    const int64_t ni = nitems(i), nn = int64_t(L.d.nnx) * L.d.nny * L.d.nnz;
    for (int64_t it = tid; it < ni; it += nthreads) {
      int a, b, c, r;
      int64_t n;
      dof_item(it, L.d, a, b, c, r, n);
      if (n >= nn) continue;
      const int64_t dof = 3 * n + r;
      const float s = stencil_row<float, true>(L.d, L.A, xin, a, b, c, r);
      rout[dof] = L.act[dof] ? __ldcg(L.b + dof) - s : 0.0f;
    }
  };
  // Level i's residual restricted into level i + 1's right-hand side, and --
  // for a smoothed level -- its first smoothing step from zero, per DOF.
  auto restrict_to = [&](int i) {
    const FusedLevel& F = fc.L[i];
    const FusedLevel& C = fc.L[i + 1];
    const float* rf = O(i);
    const bool smoothed = i + 1 < top;
    const int64_t nn = int64_t(C.d.nnx) * C.d.nny * C.d.nnz;
    float* xfirst = C.xq;  // Chebyshev step 0 writes the other buffer (x = 0 in xp)
    if (smoothed && fc.cheb_m == 0) xfirst = C.xp;  // Jacobi's first sweep writes the iterate
    for (int64_t n = tid; n < nn; n += nthreads) {
      int a, b, c;
      node_abc(C.d, n, a, b, c);
      float s[3];
      restrict_node<float, true>(F.d, C.d, rf, a, b, c, s);
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const int64_t dof = 3 * n + k;
        const float bv = C.act[dof] ? s[k] : 0.0f;
        C.b[dof] = bv;
        if (!smoothed) continue;
        if (fc.cheb_m > 0) {
          const float dn = C.act[dof] ? C.coef[0] * (C.dinv[dof] * (bv - 0.0f)) : 0.0f;
          C.chd[dof] = dn;
          xfirst[dof] = C.act[dof] ? 0.0f + dn : 0.0f;
        } else {
          xfirst[dof] = fc.omega * C.dinv[dof] * bv;
        }
      }
    }
    if (smoothed && fc.cheb_m > 0) cur[i + 1] = 1;
  };
  auto prolong_from = [&](int i) {  // level i's iterate += P (level i + 1's iterate)
    const FusedLevel& F = fc.L[i];
    const FusedLevel& C = fc.L[i + 1];
    const float* ec = X(i + 1);
    float* xf = X(i);
    const int64_t nn = int64_t(F.d.nnx) * F.d.nny * F.d.nnz;
    for (int64_t n = tid; n < nn; n += nthreads) {
      int a, b, c;
      node_abc(F.d, n, a, b, c);
      float s[3];
      prolong_node<float, true>(F.d, C.d, ec, a, b, c, s);
#pragma unroll
      for (int k = 0; k < 3; ++k)
        if (F.act[3 * n + k]) xf[3 * n + k] = __ldcg(xf + 3 * n + k) + s[k];
    }
  };
  auto coarsest = [&]() {  // x = A^-1 b over the compact numbering, a warp per row
    const FusedLevel& L = fc.L[top];
    const int64_t ndof = 3 * int64_t(L.d.nnx) * L.d.nny * L.d.nnz;
    for (int64_t dd = tid; dd < ndof; dd += nthreads)
      if (fc.cidx[dd] < 0) L.xp[dd] = 0.0f;
    const int lane = threadIdx.x & 31;
    const int64_t warp = tid >> 5, nwarps = nthreads >> 5;
    for (int64_t row = warp; row < fc.nc; row += nwarps) {
      double s = 0.0;
      for (int k = lane; k < fc.nc; k += 32)
        s += fc.Ainv[row * fc.nc + k] * double(__ldcg(L.b + fc.cdof[k]));
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
      if (lane == 0) L.xp[fc.cdof[row]] = float(s);
    }
    cur[top] = 0;
  };

  // Down: level 0's first step from zero (its right-hand side came from level 1).
  smooth(0, 0, true);
  cluster_sync_all();
  for (int i = 0; i < top; ++i) {
    const int steps = fc.cheb_m > 0 ? fc.cheb_m : fc.sweeps;
    for (int k = 1; k < steps; ++k) {
      smooth(i, k, false);
      cluster_sync_all();
    }
    residual(i);
    cluster_sync_all();
    restrict_to(i);
    cluster_sync_all();
  }
  coarsest();
  for (int i = top - 1; i >= 0; --i) {
    cluster_sync_all();
    prolong_from(i);
    const int steps = fc.cheb_m > 0 ? fc.cheb_m : fc.sweeps;
    for (int k = 0; k < steps; ++k) {
      cluster_sync_all();
      smooth(i, k, false);
    }
  }
}

}  // namespace

// Cluster size of the fused launch: the largest of 16 (non-portable), 8, 4, 2
// CTAs that the device can co-schedule with this kernel's resources.
int fused_coarse_blocks() {
  static std::atomic<int> cached{0};
  const int c = cached.load();
  if (c > 0) return c;
  TG_CUDA(cudaFuncSetAttribute(k_coarse_vcycle, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
  int best = 1;
  for (int cs : {16, 8, 4, 2}) {
    cudaLaunchConfig_t cfg{};
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = unsigned(cs);
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(unsigned(cs));
    cfg.blockDim = dim3(kFusedThreads);
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int n = 0;
    if (cudaOccupancyMaxActiveClusters(&n, k_coarse_vcycle, &cfg) == cudaSuccess && n >= 1) {
      best = cs;
      break;
    }
    cudaGetLastError();  // an unsupported size is not an error of the solve
  }
  cached.store(best);
  return best;
}

void mg_coarse_vcycle_fused(const FusedCoarse& fc, cudaStream_t s) {
  const int cs = fused_coarse_blocks();
  cudaLaunchConfig_t cfg{};
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = unsigned(cs);
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.gridDim = dim3(unsigned(cs));
  cfg.blockDim = dim3(kFusedThreads);
  cfg.stream = s;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  TG_CUDA(cudaLaunchKernelEx(&cfg, k_coarse_vcycle, fc));
  note_launch();
}

}  // namespace tg
