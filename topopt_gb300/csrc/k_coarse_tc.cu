// k_coarse_tc.cu -- the level-1 Galerkin operator of the FP32 V-cycle on the
// tensor cores (tcgen05, TMEM accumulators).
//
// Reference counterpart: the level-1 operator A1 = P0^T A0 P0 of the matrix-free
// hierarchy (core/src/fea/multigrid.cpp:1413-1446, galerkin_a1_from_prolong
// :1543-1899), applied by v_cycle's jacobi_sweep and residual (:780-817) as an
// Eigen SpMV.  Here it is applied without an assembled matrix.
//
// A coarse element's matrix is the sum over its eight children c of
// W_c^T (E_c Ke) W_c.  Where every DOF involved is active (all but the elements
// touching Dirichlet DOFs, voids' untouched DOFs or an odd axis's last half
// element) this is sum_c E_c G_c with the eight fixed 24x24 blocks
// G_c = W_c^T Ke W_c.  For a batch of 128 coarse elements (the rows of U, one
// element's 24 DOF values per row) the tensor cores form
//     D = U [G_0 | G_1 | ... | G_7]          (M = 128, N = 192, K = 24)
// and each thread finishes its element as y = sum_c E_c D[:, 24c : 24c+24]
// (packed FP32 multiply-adds).  FP32 accuracy from TF32 tensor cores: the
// operands are split into TF32 high parts and FP32 remainders and
// D = U_hi G_hi + U_hi G_lo + U_lo G_hi (the remainders' product is below FP32
// rounding).  Elements off the fast path use their stored element matrix.
//
// Scheduling is the FP32 fine operator's column schedule (k_operator.cu): lanes
// along x (lanes 0 and 31 halo), 4 warps stacked in y with Y element rows per
// thread, a march in z; the 128 threads' elements of one row step are one MMA
// batch, and row 32w + l of D is TMEM lane 32w + l -- the lane warp w reads.
// Node sums are combined as in that kernel (y inside the thread, x across
// lanes, the warp hand-over, z), in a fixed order: deterministic.
//
// Waits on the MMA's completion are bounded; a wait that runs out sets *err
// (the host raises a device error) instead of spinning.
#include <cuda_runtime.h>

#include "tg_internal.h"
#include "tg_multigrid.h"
#include "tg_tc.h"

#include <algorithm>
#include <atomic>

namespace tg {
namespace {

constexpr int kTcY = 4;            // element rows per thread
constexpr int kTcW = 4;            // warps (4 x 32 = the MMA's 128 rows)
constexpr int kTcRows = kTcW * kTcY - 1;
constexpr int kTcN = 192;          // 8 children x 24
constexpr int kTcSbo = 6 * 128;    // 8-row group stride: 6 K chunks of 16 bytes
constexpr int kTcABytes = 16 * kTcSbo;         // 128 rows x 24 TF32
constexpr int kTcBBytes = (kTcN / 8) * kTcSbo;  // 192 rows x 24 TF32
constexpr int kTcTmemCols = 256;
constexpr uint32_t kTcMaxPolls = 1u << 22;
// Dynamic shared memory per CTA: A hi/lo, B hi/lo and alignment slack.  Large
// enough that at most two CTAs share an SM, which is what TMEM holds (2 x 256
// columns of 512).
constexpr int kTcSmem = 2 * kTcABytes + 2 * kTcBBytes + 1024 + 40 * 1024;

__device__ __forceinline__ int kmaj(int row, int k) {
  return (row >> 3) * kTcSbo + (k >> 2) * 128 + (row & 7) * 16 + (k & 3) * 4;
}

__device__ __forceinline__ float shdn(float v) { return __shfl_down_sync(0xffffffffu, v, 1); }
__device__ __forceinline__ float shup(float v) { return __shfl_up_sync(0xffffffffu, v, 1); }

template <int MODE>
__global__ void __launch_bounds__(128) k_level1_tc(
    MgDims fd, MgDims cd, int KZ, const float* __restrict__ ef, const uint8_t* __restrict__ act,
    const int* __restrict__ spos, const float* __restrict__ yspec,
    const float* __restrict__ G, const float* __restrict__ x, const float* __restrict__ b,
    const float* __restrict__ invdiag, float omega, float* __restrict__ y,
    int* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char dsm[];
  unsigned char* base =
      dsm + ((1024 - (static_cast<uint32_t>(__cvta_generic_to_shared(dsm)) & 1023)) & 1023);
  unsigned char* a_hi = base;
  unsigned char* a_lo = base + kTcABytes;
  unsigned char* b_hi = base + 2 * kTcABytes;
  unsigned char* b_lo = base + 2 * kTcABytes + kTcBBytes;
  __shared__ float xs[2][kTcW][6][32];
  __shared__ uint64_t bar;
  __shared__ uint32_t tbase;
  constexpr int Y = kTcY, W = kTcW;
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;

  if (w == 0) {
    tc::tmem_alloc(&tbase, kTcTmemCols);
    tc::tmem_relinquish();
  }
  if (t == 0) {
    tc::mbar_init(&bar, 1);
    tc::fence_mbar_init();
  }
  // B = the 8 child blocks, row n = 24c + r holds row r of G_c (K = 24
  // columns; G_c is symmetric), split into TF32 high parts and remainders.
  for (int e = t; e < kTcN * 24; e += 128) {
    const int n = e / 24, k = e % 24;
    const float v = G[e];
    const float h = tc::tf32_hi(v);
    *reinterpret_cast<float*>(b_hi + kmaj(n, k)) = h;
    *reinterpret_cast<float*>(b_lo + kmaj(n, k)) = v - h;
  }
  tc::fence_async_smem();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tbase;
  const uint32_t idesc = tc::idesc_tf32(128, kTcN);
  uint32_t phase = 0;
  bool tc_ok = true;

  const int ex = blockIdx.x * 30 - 1 + lane;
  const int ey0 = blockIdx.y * kTcRows - 1 + w * Y;
  const int z0 = blockIdx.z * KZ;
  const int64_t plane = int64_t(cd.nnx) * cd.nny;
  const bool vx = ex >= 0 && ex < cd.nnx;
  const bool own_x = lane >= 1 && lane <= 30 && ex < cd.nnx;
  bool rv[Y + 1], ro[Y + 1], ev[Y];
#pragma unroll
  for (int i = 0; i <= Y; ++i) {
    rv[i] = vx && ey0 + i >= 0 && ey0 + i < cd.nny;
    ro[i] = own_x && i >= 1 && (i < Y || w < W - 1) && ey0 + i < cd.nny;
  }
#pragma unroll
  for (int j = 0; j < Y; ++j) ev[j] = ex >= 0 && ex < cd.ex && ey0 + j >= 0 && ey0 + j < cd.ey;
  const int64_t col = int64_t(ey0) * cd.nnx + ex;

  auto load_layer = [&](int c, float (&r)[Y + 1][3]) {
    const bool vc = c >= 0 && c < cd.nnz;
    const float* p = x + 3 * (int64_t(c) * plane + col);
#pragma unroll
    for (int i = 0; i <= Y; ++i)
#pragma unroll
      for (int k = 0; k < 3; ++k) r[i][k] = (vc && rv[i]) ? p[3 * i * cd.nnx + k] : 0.0f;
  };

  float cur[Y + 1][3], nxt[Y + 1][3], raw[Y + 1][3];
  load_layer(z0 - 1, cur);
  load_layer(z0, nxt);
  float pend[Y + 1][3];
#pragma unroll
  for (int i = 0; i <= Y; ++i) pend[i][0] = pend[i][1] = pend[i][2] = 0.0f;

  // Activity, right-hand side and inverse diagonal of node row i, layer c,
  // requested an element ahead of their use.
  struct RowIn {
    float bv[3], dv[3];
    bool ak[3];
  };
  auto load_row = [&](int i, int c, RowIn& q) {
    const bool ok = c >= 0 && c < cd.nnz && ro[i];
    const int64_t d0 = 3 * (int64_t(c) * plane + col + int64_t(i) * cd.nnx);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      q.ak[k] = ok && act[d0 + k] != 0;
      q.bv[k] = (MODE != kApply && ok) ? b[d0 + k] : 0.0f;
      q.dv[k] = (MODE == kSmooth && ok) ? invdiag[d0 + k] : 0.0f;
    }
  };
  auto emit = [&](int i, int ez, const float (&ax)[3], const RowIn& q) {
    const int64_t d0 = 3 * (int64_t(ez) * plane + col + int64_t(i) * cd.nnx);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      float out;
      if (!q.ak[k]) {
        out = 0.0f;
      } else if constexpr (MODE == kApply) {
        out = ax[k];
      } else if constexpr (MODE == kResidual) {
        out = q.bv[k] - ax[k];
      } else {
        out = cur[i][k] + omega * q.dv[k] * (q.bv[k] - ax[k]);
      }
      y[d0 + k] = out;
    }
  };

#pragma unroll 1
  for (int s = 0; s <= KZ; ++s) {
    const int ez = z0 - 1 + s;
    if (s < KZ) load_layer(ez + 2, raw);
    const bool out_z = s >= 1 && ez < cd.nnz;
    const bool ezok = ez >= 0 && ez < cd.ez;
    RowIn rin;
    load_row(1, out_z ? ez : -1, rin);
    float c1[3], n1[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      c1[k] = shdn(cur[0][k]);
      n1[k] = shdn(nxt[0][k]);
    }
    float C[2][2][3];
#pragma unroll
    for (int j = 0; j < Y; ++j) {
      float c1u[3], n1u[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        c1u[k] = shdn(cur[j + 1][k]);
        n1u[k] = shdn(nxt[j + 1][k]);
      }
      // The element's 24 DOF values, corner c = xb | yb << 1 | zb << 2.
      float u[24];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        u[0 * 3 + k] = cur[j][k];
        u[1 * 3 + k] = c1[k];
        u[2 * 3 + k] = cur[j + 1][k];
        u[3 * 3 + k] = c1u[k];
        u[4 * 3 + k] = nxt[j][k];
        u[5 * 3 + k] = n1[k];
        u[6 * 3 + k] = nxt[j + 1][k];
        u[7 * 3 + k] = n1u[k];
      }
      const bool valid = ev[j] && ezok;
      const int64_t ce = valid ? (int64_t(ez) * cd.ey + (ey0 + j)) * cd.ex + ex : 0;
      const int sp = valid ? spos[ce] : -1;  // off the fast path: its outputs precomputed
      // Children's moduli (0 for children outside the fine grid).
      float E[8];
#pragma unroll
      for (int c = 0; c < 8; ++c) {
        const int fi = 2 * ex + (c & 1), fj = 2 * (ey0 + j) + ((c >> 1) & 1),
                  fk = 2 * ez + (c >> 2);
        E[c] = (valid && fi < fd.ex && fj < fd.ey && fk < fd.ez)
                   ? ef[(int64_t(fk) * fd.ey + fj) * fd.ex + fi]
                   : 0.0f;
      }
      // Row 32w + lane of the batch's U, high parts and remainders.
#pragma unroll
      for (int q = 0; q < 6; ++q) {
        float4 h, l;
        h.x = tc::tf32_hi(u[4 * q + 0]); l.x = u[4 * q + 0] - h.x;
        h.y = tc::tf32_hi(u[4 * q + 1]); l.y = u[4 * q + 1] - h.y;
        h.z = tc::tf32_hi(u[4 * q + 2]); l.z = u[4 * q + 2] - h.z;
        h.w = tc::tf32_hi(u[4 * q + 3]); l.w = u[4 * q + 3] - h.w;
        *reinterpret_cast<float4*>(a_hi + kmaj(t, 4 * q)) = h;
        *reinterpret_cast<float4*>(a_lo + kmaj(t, 4 * q)) = l;
      }
      tc::fence_async_smem();
      tc::fence_before_sync();
      __syncthreads();
      if (t == 0) {
        tc::fence_after_sync();
        const unsigned char* as[3] = {a_hi, a_hi, a_lo};
        const unsigned char* bs[3] = {b_hi, b_lo, b_hi};
#pragma unroll
        for (int p = 0; p < 3; ++p)
#pragma unroll
          for (int kk = 0; kk < 3; ++kk) {
            const uint64_t da = tc::smem_desc(tc::smem_u32(as[p] + kk * 256), 128, kTcSbo);
            const uint64_t db = tc::smem_desc(tc::smem_u32(bs[p] + kk * 256), 128, kTcSbo);
            tc::mma_tf32(tmem, da, db, idesc, (p | kk) ? 1u : 0u);
          }
        tc::mma_commit(&bar);
      }
      const bool got = tc::mbar_wait(&bar, phase, kTcMaxPolls);
      phase ^= 1u;
      tc::fence_after_sync();
      if (!got && tc_ok) {
        tc_ok = false;
        atomicExch(err, 1);
      }
      // y = sum_c E_c D[:, 24c : 24c + 24], or the stored matrix off the fast path.
      float2 acc[12];
#pragma unroll
      for (int r = 0; r < 12; ++r) acc[r] = make_float2(0.0f, 0.0f);
      if (tc_ok) {
#pragma unroll
        for (int q = 0; q < kTcN / 32; ++q) {
          float v[32];
          tc::tmem_ld32(tmem + (uint32_t(32 * w) << 16) + uint32_t(32 * q), v);
          tc::tmem_ld_wait();
#pragma unroll
          for (int i = 0; i < 32; i += 2) {
            const int cl = 32 * q + i, ch = cl / 24, r = cl % 24;
            acc[r / 2] = __ffma2_rn(make_float2(v[i], v[i + 1]), make_float2(E[ch], E[ch]),
                                    acc[r / 2]);
          }
        }
      }
      tc::fence_before_sync();
      float out[24];
#pragma unroll
      for (int r = 0; r < 12; ++r) {
        out[2 * r] = acc[r].x;
        out[2 * r + 1] = acc[r].y;
      }
      if (sp >= 0) {
#pragma unroll
        for (int r = 0; r < 24; ++r) out[r] = yspec[int64_t(sp) * 24 + r];
      }
      // Node row j: the previous element's +y corners and this element's -y
      // corners, then the x-combine with the lane below.
      float T[2][2][3];
#pragma unroll
      for (int cx = 0; cx < 2; ++cx)
#pragma unroll
        for (int cz = 0; cz < 2; ++cz) {
          const int c0 = cx | (cz << 2), c1i = cx | 2 | (cz << 2);
#pragma unroll
          for (int k = 0; k < 3; ++k) {
            T[cx][cz][k] = j > 0 ? C[cx][cz][k] + out[3 * c0 + k] : out[3 * c0 + k];
            C[cx][cz][k] = out[3 * c1i + k];
          }
        }
      float N[2][3];
#pragma unroll
      for (int cz = 0; cz < 2; ++cz)
#pragma unroll
        for (int k = 0; k < 3; ++k) N[cz][k] = T[0][cz][k] + shup(T[1][cz][k]);
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
        if (out_z && ro[j]) emit(j, ez, ax, rin);
        load_row(j + 1, out_z ? ez : -1, rin);
      }
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        c1[k] = c1u[k];
        n1[k] = n1u[k];
      }
    }
    float NY[2][3];
#pragma unroll
    for (int cz = 0; cz < 2; ++cz)
#pragma unroll
      for (int k = 0; k < 3; ++k) NY[cz][k] = C[0][cz][k] + shup(C[1][cz][k]);
    __syncthreads();
    if (w < W - 1) {
      float ax[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        ax[k] = pend[Y][k] + (NY[0][k] + xs[s & 1][w + 1][k][lane]);
        pend[Y][k] = NY[1][k] + xs[s & 1][w + 1][3 + k][lane];
      }
      if (out_z && ro[Y]) emit(Y, ez, ax, rin);
    }
#pragma unroll
    for (int i = 0; i <= Y; ++i)
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        cur[i][k] = nxt[i][k];
        nxt[i][k] = raw[i][k];
      }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (w == 0) tc::tmem_dealloc(tmem, kTcTmemCols);
}

// The elements off the fast path: one warp per element, lane r < 24 forms row r
// of (stored element matrix) x (element DOFs) into yspec[p].
__global__ void __launch_bounds__(256) k_level1_special(MgDims cd, int nspec,
                                                        const int* __restrict__ list,
                                                        const float* __restrict__ Kel,
                                                        const float* __restrict__ x,
                                                        float* __restrict__ yspec) {
  const int lane = threadIdx.x & 31;
  const int p = blockIdx.x * 8 + (threadIdx.x >> 5);
  if (p >= nspec) return;
  const int64_t ce = list[p];
  const int I = int(ce % cd.ex), J = int((ce / cd.ex) % cd.ey), K = int(ce / (int64_t(cd.ex) * cd.ey));
  float uk = 0.0f;
  if (lane < 24) {
    const int c = lane / 3, comp = lane % 3;
    const int64_t node = (int64_t(K + (c >> 2)) * cd.nny + (J + ((c >> 1) & 1))) * cd.nnx +
                         (I + (c & 1));
    uk = x[3 * node + comp];
  }
  float a = 0.0f;
  const float* Kr = Kel + ce * 576 + int64_t(lane < 24 ? lane : 0) * 24;
#pragma unroll
  for (int k = 0; k < 24; ++k) a = fmaf(Kr[k], __shfl_sync(0xffffffffu, uk, k), a);
  if (lane < 24) yspec[int64_t(p) * 24 + lane] = a;
}

}  // namespace

// z-chunks of about 6 node layers: enough CTAs to fill the GPU at two per SM.
int level1_tc_kz(const MgDims& cd) {
  const int chunks = std::max(1, (cd.nnz + 5) / 6);
  return std::max(4, (cd.nnz + chunks - 1) / chunks);
}

void mg_level1_tc(int mode, const MgDims& fd, const MgDims& cd, const float* ef,
                  const uint8_t* act, const int* spos, const int* slist, int nspec,
                  const float* Kel, const float* G, const float* x, const float* b,
                  const float* invdiag, float omega, float* y, float* yspec, int* err,
                  cudaStream_t s) {
  static std::atomic<int> attr_set{0};  // the attribute is set once per process
  if (!attr_set.load()) {
    TG_CUDA(cudaFuncSetAttribute(k_level1_tc<kApply>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 kTcSmem));
    TG_CUDA(cudaFuncSetAttribute(k_level1_tc<kResidual>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem));
    TG_CUDA(cudaFuncSetAttribute(k_level1_tc<kSmooth>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem));
    attr_set.store(1);
  }
  if (nspec > 0) {
    k_level1_special<<<(nspec + 7) / 8, 256, 0, s>>>(cd, nspec, slist, Kel, x, yspec);
    TG_LAUNCH_CHECK();
  }
  const int kz = level1_tc_kz(cd);
  const dim3 grid((cd.nnx + 29) / 30, (cd.nny + kTcRows - 1) / kTcRows, (cd.nnz + kz - 1) / kz);
  if (mode == kApply)
    k_level1_tc<kApply><<<grid, 128, kTcSmem, s>>>(fd, cd, kz, ef, act, spos, yspec, G, x, b,
                                                   invdiag, omega, y, err);
  else if (mode == kResidual)
    k_level1_tc<kResidual><<<grid, 128, kTcSmem, s>>>(fd, cd, kz, ef, act, spos, yspec, G, x, b,
                                                      invdiag, omega, y, err);
  else
    k_level1_tc<kSmooth><<<grid, 128, kTcSmem, s>>>(fd, cd, kz, ef, act, spos, yspec, G, x, b,
                                                    invdiag, omega, y, err);
  TG_LAUNCH_CHECK();
}

}  // namespace tg
