// homog.cu -- periodic strain homogenization of batches of unit cells.
//
// Reference counterpart: homogenize() of the lattice harness
// (core/tests/harness/lattice_homog_probe.cpp:290-412).  For each cell (a
// nx*ny*nz voxel grid on the torus: opposite faces identified) and each Voigt
// unit strain J in [xx, yy, zz, gxy, gyz, gzx] (engineering shear):
//   F_J = sum_e ke chi0_J                       (chi0: element nodal displacement
//                                                of the unit strain, :240-265)
//   K chi_J = F_J                               (node 0's DOFs and DOFs touched by
//                                                no solid element pinned)
//   CH[I][J] = (1/|Y|) sum_e chi0_I^T ke (chi0_J - chi_J,e)
// solved by Jacobi-preconditioned CG (the harness's Eigen ConjugateGradient with
// its default diagonal preconditioner and stop test |r|^2 < tol^2 |b|^2).
//
// GPU layout: every (cell, strain) pair is one system of the batch; all systems
// advance in lock step through the batched periodic operator (k_operator.cu,
// PER instantiation) and batched vector kernels with per-system scalars, and a
// converged system freezes (its own iteration count and iterate are exactly what
// a solo solve would give).  Mixed precision: FP64 iterative refinement (FP64
// residual b - A x) around lock-step FP32 Jacobi-PCG inner solves on the
// unit-norm residual, FP64 dot products throughout.  The CH sum is evaluated as
//   CH[I][J] = (n_solid chi0_I^T ke chi0_J - F_I . chi_J) / |Y|,
// the same sum regrouped: sum_e chi0_I^T ke chi_J,e = F_I . chi_J.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

#include "tg_solver.h"

namespace tg {
namespace {

constexpr int kT = 256;

// Hex8 local corner offsets (reference node order, hex_element.cpp).
constexpr int kHexOff[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                               {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};

struct CornerLoads {
  double fe[6][8][3];  // (ke chi0_J) at corner a, component c, unit modulus
};

// The same offsets as bit arithmetic, for device code.
__device__ __forceinline__ int hex_ox(int a) { return ((a + 1) >> 1) & 1; }
__device__ __forceinline__ int hex_oy(int a) { return (a >> 1) & 1; }
__device__ __forceinline__ int hex_oz(int a) { return a >> 2; }

__device__ __forceinline__ int dwrap(int a, int n) {
  a %= n;
  return a < 0 ? a + n : a;
}

// Per cell and node: element factors, kept mask, inverse diagonal and the six
// right-hand sides (zero on pinned DOFs).  Sums run over the corners in a fixed
// order, so the fields are deterministic.
__global__ void k_homog_cell(const uint8_t* __restrict__ tags, int ncell, int nx, int ny, int nz,
                             double E, double kdiag, CornerLoads cl, double* __restrict__ ef,
                             uint8_t* __restrict__ kept, double* __restrict__ invd,
                             double* __restrict__ F) {
  const int64_t np = int64_t(nx) * ny * nz, nd = 3 * np;
  const int64_t total = np * ncell;
  for (int64_t q = blockIdx.x * int64_t(kT) + threadIdx.x; q < total;
       q += int64_t(gridDim.x) * kT) {
    const int64_t cell = q / np, p = q - cell * np;
    const int i = int(p % nx), j = int((p / nx) % ny), k = int(p / (int64_t(nx) * ny));
    const uint8_t* tg = tags + cell * np;
    ef[q] = tg[p] ? E : 0.0;
    int cnt = 0;
    double f[6][3];
#pragma unroll
    for (int J = 0; J < 6; ++J) f[J][0] = f[J][1] = f[J][2] = 0.0;
#pragma unroll
    for (int a = 0; a < 8; ++a) {
      // The element whose corner a is node p.
      const int ei = dwrap(i - hex_ox(a), nx), ej = dwrap(j - hex_oy(a), ny),
                ek = dwrap(k - hex_oz(a), nz);
      if (!tg[(int64_t(ek) * ny + ej) * nx + ei]) continue;
      ++cnt;
#pragma unroll
      for (int J = 0; J < 6; ++J)
#pragma unroll
        for (int c = 0; c < 3; ++c) f[J][c] += cl.fe[J][a][c];
    }
    for (int c = 0; c < 3; ++c) {
      const int64_t d = 3 * p + c;
      const bool kk = cnt > 0 && d >= 3;  // node 0 pinned, untouched DOFs pinned
      kept[cell * nd + d] = kk;
      invd[cell * nd + d] = kk ? 1.0 / (kdiag * E * double(cnt)) : 0.0;
#pragma unroll
      for (int J = 0; J < 6; ++J) F[(cell * 6 + J) * nd + d] = kk ? f[J][c] : 0.0;
    }
  }
}

// Batched reductions: system bi's partials are written by the CTAs of grid row
// blockIdx.y, each over a fixed slice; k_bsum adds them in a fixed order.
__device__ __forceinline__ double bred(double v, double* sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  double s = 0.0;
  if (wid == 0) {
    s = lane < (kT >> 5) ? sh[lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  }
  return s;
}

// rr = r.r, rz = r.(D^-1 r) per system.
template <class T>
__global__ void k_b_rr_rz(const T* __restrict__ R, const T* __restrict__ invd, int64_t nd,
                          int nrhs, double* __restrict__ prr, double* __restrict__ prz) {
  __shared__ double sh[32];
  const int bi = blockIdx.y, P = gridDim.x;
  const T* r = R + bi * nd;
  const T* iv = invd + (bi / nrhs) * nd;
  double a = 0.0, b = 0.0;
  for (int64_t d = blockIdx.x * int64_t(kT) + threadIdx.x; d < nd; d += int64_t(P) * kT) {
    const double v = double(r[d]);
    a += v * v;
    b += v * (double(iv[d]) * v);
  }
  a = bred(a, sh);
  b = bred(b, sh);
  if (threadIdx.x == 0) {
    prr[int64_t(bi) * P + blockIdx.x] = a;
    prz[int64_t(bi) * P + blockIdx.x] = b;
  }
}

// One warp per system: out[bi] = sum of its P partials, in order.
__global__ void k_bsum(const double* __restrict__ part, int P, int B, double* __restrict__ out,
                       const double* __restrict__ part2, double* __restrict__ out2) {
  const int bi = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (bi >= B) return;
  double s = 0.0, s2 = 0.0;
  for (int q = lane; q < P; q += 32) {
    s += part[int64_t(bi) * P + q];
    if (part2) s2 += part2[int64_t(bi) * P + q];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    s += __shfl_down_sync(0xffffffffu, s, o);
    s2 += __shfl_down_sync(0xffffffffu, s2, o);
  }
  if (lane == 0) {
    out[bi] = s;
    if (part2) out2[bi] = s2;
  }
}

// Start: Bv = R = F[cell][J], X = 0.
__global__ void k_b_start(const double* __restrict__ F, const int* __restrict__ jlist, int64_t nd,
                          int nrhs, double* __restrict__ Bv, double* __restrict__ X,
                          double* __restrict__ R) {
  const int bi = blockIdx.y;
  const int cell = bi / nrhs, J = jlist[bi - cell * nrhs];
  const double* f = F + (int64_t(cell) * 6 + J) * nd;
  for (int64_t d = blockIdx.x * int64_t(kT) + threadIdx.x; d < nd;
       d += int64_t(gridDim.x) * kT) {
    const double r = f[d];
    Bv[bi * nd + d] = r;
    X[bi * nd + d] = 0.0;
    R[bi * nd + d] = r;
  }
}

// Inner start of system bi when it runs (run[bi] != 0): X = 0, P = D^-1 R;
// with a scale (mixed form) R is first set to float(r64 / |r64|).
template <class T>
__global__ void k_b_begin(const double* __restrict__ r64, const double* __restrict__ rn,
                          const T* __restrict__ invd, int64_t nd, int nrhs,
                          const int* __restrict__ run, T* __restrict__ X, T* __restrict__ R,
                          T* __restrict__ Pv) {
  const int bi = blockIdx.y;
  if (run && !run[bi]) return;
  const T* iv = invd + (bi / nrhs) * nd;
  const double inv = r64 ? 1.0 / rn[bi] : 1.0;
  for (int64_t d = blockIdx.x * int64_t(kT) + threadIdx.x; d < nd;
       d += int64_t(gridDim.x) * kT) {
    const T r = r64 ? T(r64[bi * nd + d] * inv) : R[bi * nd + d];
    R[bi * nd + d] = r;
    X[bi * nd + d] = T(0);
    Pv[bi * nd + d] = iv[d] * r;
  }
}

// Per-system CG state: act 1 = iterating, 0 = converged, 2 = stopped
// (iteration budget or breakdown), -1 = not run (run[bi] == 0).
__global__ void k_b_init(int B, const double* __restrict__ rr, const double* __restrict__ rz,
                         double tol, const int* __restrict__ run, int* __restrict__ act,
                         int* __restrict__ it, double* __restrict__ thr,
                         double* __restrict__ rhs2, double* __restrict__ absn) {
  const int bi = blockIdx.x * blockDim.x + threadIdx.x;
  if (bi >= B) return;
  it[bi] = 0;
  if (run && !run[bi]) {
    act[bi] = -1;
    return;
  }
  const double b2 = rr[bi];
  double t = tol * tol * b2;
  if (t < DBL_MIN) t = DBL_MIN;
  thr[bi] = t;
  rhs2[bi] = b2;
  absn[bi] = rz[bi];
  act[bi] = (b2 > 0.0 && !(b2 < t)) ? 1 : 0;
}

// x += alpha p, r -= alpha t for iterating systems (alpha = absNew / p.Ap), with
// the partials of r.r and r.(D^-1 r) of the updated residual.
template <class T>
__global__ void k_b_xr(T* __restrict__ X, T* __restrict__ R, const T* __restrict__ Pv,
                       const T* __restrict__ Tv, const T* __restrict__ invd, int64_t nd, int nrhs,
                       const double* __restrict__ absn, const double* __restrict__ pap,
                       const int* __restrict__ act, double* __restrict__ prr,
                       double* __restrict__ prz) {
  __shared__ double sh[32];
  const int bi = blockIdx.y, P = gridDim.x;
  double a = 0.0, b = 0.0;
  if (act[bi] == 1) {
    const double pa = pap[bi];
    const T alpha = T(pa > 0.0 ? absn[bi] / pa : 0.0);
    const T* iv = invd + (bi / nrhs) * nd;
    T* x = X + bi * nd;
    T* r = R + bi * nd;
    const T* p = Pv + bi * nd;
    const T* t = Tv + bi * nd;
    for (int64_t d = blockIdx.x * int64_t(kT) + threadIdx.x; d < nd; d += int64_t(P) * kT) {
      x[d] += alpha * p[d];
      const T v = r[d] - alpha * t[d];
      r[d] = v;
      const double vd = double(v);
      a += vd * vd;
      b += vd * (double(iv[d]) * vd);
    }
  }
  a = bred(a, sh);
  b = bred(b, sh);
  if (threadIdx.x == 0) {
    prr[int64_t(bi) * P + blockIdx.x] = a;
    prz[int64_t(bi) * P + blockIdx.x] = b;
  }
}

// The scalar step of every iterating system: stop at the threshold (this
// iteration not counted, as Eigen), else beta = rz / absNew, absNew = rz, one
// more iteration, and stop at the budget.  nact counts the systems still iterating.
__global__ void k_b_scalars(int B, const double* __restrict__ rr, const double* __restrict__ rz,
                            const double* __restrict__ thr, const double* __restrict__ pap,
                            int max_it, int* __restrict__ act, int* __restrict__ it,
                            double* __restrict__ absn, double* __restrict__ beta,
                            int* __restrict__ nact) {
  const int bi = blockIdx.x * blockDim.x + threadIdx.x;
  if (bi >= B || act[bi] != 1) return;
  if (!(pap[bi] > 0.0)) {
    act[bi] = 2;  // breakdown: p.Ap <= 0
    return;
  }
  if (rr[bi] < thr[bi]) {
    act[bi] = 0;
    return;
  }
  beta[bi] = rz[bi] / absn[bi];
  absn[bi] = rz[bi];
  const int n = it[bi] + 1;
  it[bi] = n;
  if (n >= max_it) {
    act[bi] = 2;
    return;
  }
  atomicAdd(nact, 1);
}

// p = D^-1 r + beta p for iterating systems.
template <class T>
__global__ void k_b_p(T* __restrict__ Pv, const T* __restrict__ R, const T* __restrict__ invd,
                      int64_t nd, int nrhs, const double* __restrict__ beta,
                      const int* __restrict__ act) {
  const int bi = blockIdx.y;
  if (act[bi] != 1) return;
  const T bt = T(beta[bi]);
  const T* iv = invd + (bi / nrhs) * nd;
  T* p = Pv + bi * nd;
  const T* r = R + bi * nd;
  for (int64_t d = blockIdx.x * int64_t(kT) + threadIdx.x; d < nd;
       d += int64_t(gridDim.x) * kT)
    p[d] = iv[d] * r[d] + bt * p[d];
}

// Mixed form: X64 += |r| * X32 for the systems that ran.
__global__ void k_b_correct(double* __restrict__ X, const float* __restrict__ Xf,
                            const double* __restrict__ rn, const int* __restrict__ run,
                            int64_t nd) {
  const int bi = blockIdx.y;
  if (!run[bi]) return;
  const double sc = rn[bi];
  for (int64_t d = blockIdx.x * int64_t(kT) + threadIdx.x; d < nd;
       d += int64_t(gridDim.x) * kT)
    X[bi * nd + d] += sc * double(Xf[bi * nd + d]);
}

// Refinement bookkeeping per system: run the inner solve when the FP64
// residual is above the threshold; rn = |r|.
__global__ void k_b_refine(int B, const double* __restrict__ rr, const double* __restrict__ thr,
                           int* __restrict__ run, double* __restrict__ rn,
                           int* __restrict__ nrun) {
  const int bi = blockIdx.x * blockDim.x + threadIdx.x;
  if (bi >= B) return;
  const double v = rr[bi];
  const int go = (v >= thr[bi] && v > 0.0 && isfinite(v)) ? 1 : 0;
  run[bi] = go;
  rn[bi] = sqrt(v);
  if (go) atomicAdd(nrun, 1);
}

__global__ void k_to_f32(const double* __restrict__ a, float* __restrict__ b, int64_t n) {
  for (int64_t i = blockIdx.x * int64_t(kT) + threadIdx.x; i < n; i += int64_t(gridDim.x) * kT)
    b[i] = float(a[i]);
}

// Partials of F[cell][I] . X[bi] for I = 0..5 (grid.z = I).
__global__ void k_b_fx(const double* __restrict__ F, const double* __restrict__ X, int64_t nd,
                       int nrhs, double* __restrict__ part) {
  __shared__ double sh[32];
  const int bi = blockIdx.y, I = blockIdx.z, P = gridDim.x;
  const int cell = bi / nrhs;
  const double* f = F + (int64_t(cell) * 6 + I) * nd;
  const double* x = X + bi * nd;
  double a = 0.0;
  for (int64_t d = blockIdx.x * int64_t(kT) + threadIdx.x; d < nd; d += int64_t(P) * kT)
    a += f[d] * x[d];
  a = bred(a, sh);
  if (threadIdx.x == 0) part[(int64_t(bi) * 6 + I) * P + blockIdx.x] = a;
}

double now_ms() {
  return std::chrono::duration<double, std::milli>(
             std::chrono::steady_clock::now().time_since_epoch())
      .count();
}

// Shapes and per-system scratch of one batched solve.
struct Batch {
  int nx, ny, nz, nrhs, B, P;
  int64_t nd;
  ModalConsts mc;
  const uint8_t* kept;
  cudaStream_t s;
  DBuf<double> prr, prz, ppap, rr, rz, pap, thr, rhs2, absn, beta, rn;
  DBuf<int> act, it, nact, run, nrun;
  int64_t iterations_total = 0;
  int iterations_max = 0;
  void init(int B_, int64_t nd_, int P_) {
    B = B_;
    nd = nd_;
    P = P_;
    const int Pop = std::max(periodic_op_blocks<double>(nx, ny, nz),
                             periodic_op_blocks<float>(nx, ny, nz));
    prr.alloc(size_t(B) * P);
    prz.alloc(size_t(B) * P);
    ppap.alloc(size_t(B) * Pop);
    for (DBuf<double>* d : {&rr, &rz, &pap, &thr, &rhs2, &absn, &beta, &rn}) d->alloc(size_t(B));
    for (DBuf<int>* d : {&act, &it, &run}) d->alloc(size_t(B));
    nact.alloc(1);
    nrun.alloc(1);
  }
  dim3 g2() const { return dim3(static_cast<unsigned>(P), static_cast<unsigned>(B)); }
  int sb() const { return (B + 255) / 256; }
  int wb() const { return (B * 32 + 255) / 256; }

  // Lock-step Jacobi-PCG on A X = R (R holds b on entry; X, P, Tv scratch);
  // systems with run[bi] == 0 (when run is given) do nothing.  With r64 the
  // right-hand side is float(r64 / rn) (the mixed inner solve).
  template <class T>
  int pcg(T* X, T* R, T* Pv, T* Tv, const T* ef, const T* invd, double tol, int max_it,
          const int* runp, const double* r64) {
    k_b_begin<T><<<g2(), kT, 0, s>>>(r64, rn.p, invd, nd, nrhs, runp, X, R, Pv);
    TG_LAUNCH_CHECK();
    k_b_rr_rz<T><<<g2(), kT, 0, s>>>(R, invd, nd, nrhs, prr.p, prz.p);
    TG_LAUNCH_CHECK();
    k_bsum<<<wb(), 256, 0, s>>>(prr.p, P, B, rr.p, prz.p, rz.p);
    TG_LAUNCH_CHECK();
    k_b_init<<<sb(), 256, 0, s>>>(B, rr.p, rz.p, tol, runp, act.p, it.p, thr.p, rhs2.p, absn.p);
    TG_LAUNCH_CHECK();
    const int Pop = periodic_op_blocks<T>(nx, ny, nz);
    int host_nact = B;
    for (int k = 0; k < max_it && host_nact > 0; ++k) {
      launch_periodic_op<T>(kApply, nx, ny, nz, mc, ef, kept, Pv, nullptr, nullptr, T(0), Tv,
                            ppap.p, B, nrhs, s);
      k_bsum<<<wb(), 256, 0, s>>>(ppap.p, Pop, B, pap.p, nullptr, nullptr);
      TG_LAUNCH_CHECK();
      k_b_xr<T><<<g2(), kT, 0, s>>>(X, R, Pv, Tv, invd, nd, nrhs, absn.p, pap.p, act.p, prr.p,
                                    prz.p);
      TG_LAUNCH_CHECK();
      k_bsum<<<wb(), 256, 0, s>>>(prr.p, P, B, rr.p, prz.p, rz.p);
      TG_LAUNCH_CHECK();
      TG_CUDA(cudaMemsetAsync(nact.p, 0, sizeof(int), s));
      k_b_scalars<<<sb(), 256, 0, s>>>(B, rr.p, rz.p, thr.p, pap.p, max_it, act.p, it.p, absn.p,
                                       beta.p, nact.p);
      TG_LAUNCH_CHECK();
      k_b_p<T><<<g2(), kT, 0, s>>>(Pv, R, invd, nd, nrhs, beta.p, act.p);
      TG_LAUNCH_CHECK();
      if ((k & 7) == 7) {
        TG_CUDA(cudaMemcpyAsync(&host_nact, nact.p, sizeof(int), cudaMemcpyDeviceToHost, s));
        TG_CUDA(cudaStreamSynchronize(s));
      }
    }
    std::vector<int> hit(static_cast<size_t>(B));
    TG_CUDA(cudaMemcpyAsync(hit.data(), it.p, sizeof(int) * B, cudaMemcpyDeviceToHost, s));
    TG_CUDA(cudaStreamSynchronize(s));
    int mx = 0;
    for (int v : hit) {
      iterations_total += v;
      mx = std::max(mx, v);
    }
    iterations_max = std::max(iterations_max, mx);
    return mx;
  }
};

}  // namespace
}  // namespace tg

extern "C" int tg_homogenize(int32_t ncell, int32_t nx, int32_t ny, int32_t nz, double spacing,
                             double youngs_modulus, double poisson, const uint8_t* tags,
                             int32_t cases_mask, double tolerance, int32_t max_iterations,
                             int32_t precision, double* ch_out, tg_homog_info* info) {
  using namespace tg;
  tg_homog_info inf;
  std::memset(&inf, 0, sizeof inf);
  const double t0 = now_ms();
  int rc = TG_OK;
  try {
    if (ncell < 1) raise(TG_EINVAL, "homogenize: ncell must be >= 1");
    if (nx < 1 || ny < 1 || nz < 1) raise(TG_EINVAL, "homogenize: cell dimensions must be >= 1");
    if (!(spacing > 0.0)) raise(TG_EINVAL, "homogenize: spacing must be > 0");
    if (!(youngs_modulus > 0.0)) raise(TG_EINVAL, "hex8_stiffness: youngs_modulus must be > 0");
    if (!(poisson > -1.0 && poisson < 0.5))
      raise(TG_EINVAL, "hex8_stiffness: poisson must be in (-1, 0.5)");
    if ((cases_mask & 0x3F) == 0 || (cases_mask & ~0x3F) != 0)
      raise(TG_EINVAL, "homogenize: cases_mask must select strain columns 0..5 (bits 0x3F)");
    if (!(tolerance > 0.0)) raise(TG_EINVAL, "homogenize: tolerance must be > 0");
    if (precision != TG_PREC_FP64 && precision != TG_PREC_MIXED)
      raise(TG_EINVAL, "homogenize: unknown precision");
    if (!tags || !ch_out) raise(TG_EINVAL, "homogenize: tags and ch_out must be non-null");
    const int64_t np = int64_t(nx) * ny * nz, nd = 3 * np;
    if (nd > (int64_t(1) << 31) - 1) raise(TG_EINVAL, "homogenize: cell too large");
    std::vector<int> jl;
    for (int J = 0; J < 6; ++J)
      if ((cases_mask >> J) & 1) jl.push_back(J);
    const int nrhs = int(jl.size());
    if (int64_t(ncell) * nrhs > 65535)
      raise(TG_EINVAL, "homogenize: at most 65535 (cell, strain) systems per call");
    const int B = ncell * nrhs;
    const int max_it = max_iterations > 0 ? max_iterations
                                          : int(std::min<int64_t>(2 * nd, 200000));
    TG_CUDA(cudaSetDevice(device_ordinal()));
    cudaStream_t s;
    TG_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    struct StreamGuard {
      cudaStream_t s;
      ~StreamGuard() { cudaStreamDestroy(s); }
    } sg{s};
    AllocScope scope(s);  // buffers below are stream-ordered on s and freed before it

    // Element matrix, chi0 and the per-corner loads (scaled by E).
    std::vector<double> ke(576);
    hex8_ke(1.0, poisson, spacing, ke.data());
    double chi0[24][6];
    std::memset(chi0, 0, sizeof chi0);
    for (int a = 0; a < 8; ++a) {
      const double X = kHexOff[a][0] * spacing, Y = kHexOff[a][1] * spacing,
                   Z = kHexOff[a][2] * spacing;
      chi0[3 * a][0] = X;
      chi0[3 * a + 1][1] = Y;
      chi0[3 * a + 2][2] = Z;
      chi0[3 * a][3] = Y;
      chi0[3 * a + 1][4] = Z;
      chi0[3 * a + 2][5] = X;
    }
    CornerLoads cl;
    double c0[6][6];
    for (int J = 0; J < 6; ++J)
      for (int r = 0; r < 24; ++r) {
        double f = 0.0;
        for (int c = 0; c < 24; ++c) f += ke[size_t(r) * 24 + c] * chi0[c][J];
        cl.fe[J][r / 3][r % 3] = youngs_modulus * f;
      }
    for (int I = 0; I < 6; ++I)
      for (int J = 0; J < 6; ++J) {
        double acc = 0.0;
        for (int r = 0; r < 24; ++r) acc += chi0[r][I] * cl.fe[J][r / 3][r % 3];
        c0[I][J] = acc;
      }
    std::vector<int64_t> nsolid(static_cast<size_t>(ncell), 0);
    for (int c = 0; c < ncell; ++c)
      for (int64_t e = 0; e < np; ++e) nsolid[size_t(c)] += tags[c * np + e] != 0;

    Batch bt;
    bt.nx = nx;
    bt.ny = ny;
    bt.nz = nz;
    bt.nrhs = nrhs;
    bt.mc = ModalConsts::make(poisson, spacing);
    bt.mc.kdiag = ke[0];
    bt.s = s;
    DBuf<uint8_t> dtags, kept;
    DBuf<double> ef, invd, F, Bv, X, R, Pv, Tv;
    dtags.alloc(size_t(ncell * np));
    TG_CUDA(cudaMemcpyAsync(dtags.p, tags, size_t(ncell * np), cudaMemcpyHostToDevice, s));
    ef.alloc(size_t(ncell * np));
    kept.alloc(size_t(ncell * nd));
    invd.alloc(size_t(ncell * nd));
    F.alloc(size_t(ncell * 6 * nd));
    for (DBuf<double>* v : {&Bv, &X, &R}) v->alloc(size_t(B) * size_t(nd));
    const int nb_cell = int(std::min<int64_t>((ncell * np + kT - 1) / kT, 152 * 64));
    k_homog_cell<<<nb_cell, kT, 0, s>>>(dtags.p, ncell, nx, ny, nz, youngs_modulus, bt.mc.kdiag,
                                         cl, ef.p, kept.p, invd.p, F.p);
    TG_LAUNCH_CHECK();
    bt.kept = kept.p;
    const int P = int(std::max<int64_t>(1, std::min<int64_t>(64, (nd + kT * 8 - 1) / (kT * 8))));
    bt.init(B, nd, P);
    DBuf<int> djl(static_cast<size_t>(B));
    std::vector<int> jl_sys(static_cast<size_t>(B));
    for (int bi = 0; bi < B; ++bi) jl_sys[size_t(bi)] = jl[size_t(bi % nrhs)];
    TG_CUDA(cudaMemcpyAsync(djl.p, jl_sys.data(), sizeof(int) * B, cudaMemcpyHostToDevice, s));
    k_b_start<<<bt.g2(), kT, 0, s>>>(F.p, djl.p, nd, nrhs, Bv.p, X.p, R.p);
    TG_LAUNCH_CHECK();
    TG_CUDA(cudaStreamSynchronize(s));
    inf.t_setup_ms = now_ms() - t0;
    const double ts = now_ms();
    bool all_ok = true;
    if (precision == TG_PREC_FP64) {
      Pv.alloc(size_t(B) * size_t(nd));
      Tv.alloc(size_t(B) * size_t(nd));
      bt.pcg<double>(X.p, R.p, Pv.p, Tv.p, ef.p, invd.p, tolerance, max_it, nullptr, nullptr);
      std::vector<double> hrr(static_cast<size_t>(B)), hb2(static_cast<size_t>(B));
      std::vector<int> hact(static_cast<size_t>(B));
      TG_CUDA(cudaMemcpyAsync(hrr.data(), bt.rr.p, sizeof(double) * B, cudaMemcpyDeviceToHost, s));
      TG_CUDA(cudaMemcpyAsync(hb2.data(), bt.rhs2.p, sizeof(double) * B, cudaMemcpyDeviceToHost, s));
      TG_CUDA(cudaMemcpyAsync(hact.data(), bt.act.p, sizeof(int) * B, cudaMemcpyDeviceToHost, s));
      TG_CUDA(cudaStreamSynchronize(s));
      for (int bi = 0; bi < B; ++bi)
        if (!(hact[size_t(bi)] == 0 &&
              (hb2[size_t(bi)] == 0.0 || std::sqrt(hrr[size_t(bi)] / hb2[size_t(bi)]) <= tolerance)))
          all_ok = false;
    } else {
      // FP64 refinement around FP32 inner solves (relative 1e-3 each).
      DBuf<float> eff32, invd32, Xf, Rf, Pf, Tf;
      eff32.alloc(size_t(ncell * np));
      invd32.alloc(size_t(ncell * nd));
      for (DBuf<float>* v : {&Xf, &Rf, &Pf, &Tf}) v->alloc(size_t(B) * size_t(nd));
      k_to_f32<<<nb_cell, kT, 0, s>>>(ef.p, eff32.p, ncell * np);
      TG_LAUNCH_CHECK();
      k_to_f32<<<nb_cell, kT, 0, s>>>(invd.p, invd32.p, ncell * nd);
      TG_LAUNCH_CHECK();
      DBuf<double> thr_o(static_cast<size_t>(B)), b2(static_cast<size_t>(B));
      // |b|^2 and the outer threshold tol^2 |b|^2.
      k_b_rr_rz<double><<<bt.g2(), kT, 0, s>>>(R.p, invd.p, nd, nrhs, bt.prr.p, bt.prz.p);
      TG_LAUNCH_CHECK();
      k_bsum<<<bt.wb(), 256, 0, s>>>(bt.prr.p, P, B, b2.p, nullptr, nullptr);
      TG_LAUNCH_CHECK();
      std::vector<double> hb2(static_cast<size_t>(B)), hthr(static_cast<size_t>(B));
      TG_CUDA(cudaMemcpyAsync(hb2.data(), b2.p, sizeof(double) * B, cudaMemcpyDeviceToHost, s));
      TG_CUDA(cudaStreamSynchronize(s));
      for (int bi = 0; bi < B; ++bi)
        hthr[size_t(bi)] = std::max(tolerance * tolerance * hb2[size_t(bi)], DBL_MIN);
      TG_CUDA(cudaMemcpyAsync(thr_o.p, hthr.data(), sizeof(double) * B, cudaMemcpyHostToDevice, s));
      std::vector<double> hrr(static_cast<size_t>(B));
      const int max_ref = 30;
      int budget = max_it;
      for (int ref = 0;; ++ref) {
        // r = b - A x (FP64) -- the first residual is b itself (x = 0).
        if (ref > 0)
          launch_periodic_op<double>(kResidual, nx, ny, nz, bt.mc, ef.p, kept.p, X.p, Bv.p,
                                     nullptr, 0.0, R.p, nullptr, B, nrhs, s);
        k_b_rr_rz<double><<<bt.g2(), kT, 0, s>>>(R.p, invd.p, nd, nrhs, bt.prr.p, bt.prz.p);
        TG_LAUNCH_CHECK();
        k_bsum<<<bt.wb(), 256, 0, s>>>(bt.prr.p, P, B, bt.rr.p, nullptr, nullptr);
        TG_LAUNCH_CHECK();
        TG_CUDA(cudaMemsetAsync(bt.nrun.p, 0, sizeof(int), s));
        k_b_refine<<<bt.sb(), 256, 0, s>>>(B, bt.rr.p, thr_o.p, bt.run.p, bt.rn.p, bt.nrun.p);
        TG_LAUNCH_CHECK();
        int nrun = 0;
        TG_CUDA(cudaMemcpyAsync(&nrun, bt.nrun.p, sizeof(int), cudaMemcpyDeviceToHost, s));
        TG_CUDA(cudaStreamSynchronize(s));
        if (nrun == 0) break;
        if (ref == max_ref || budget <= 0) {
          all_ok = false;
          break;
        }
        ++inf.refinements;
        budget -= bt.pcg<float>(Xf.p, Rf.p, Pf.p, Tf.p, eff32.p, invd32.p, 1e-3, budget, bt.run.p,
                                R.p);
        k_b_correct<<<bt.g2(), kT, 0, s>>>(X.p, Xf.p, bt.rn.p, bt.run.p, nd);
        TG_LAUNCH_CHECK();
      }
      // Converged: every final FP64 residual below its threshold (NaN fails).
      TG_CUDA(cudaMemcpyAsync(hrr.data(), bt.rr.p, sizeof(double) * B, cudaMemcpyDeviceToHost, s));
      TG_CUDA(cudaStreamSynchronize(s));
      for (int bi = 0; bi < B; ++bi)
        if (!(hrr[size_t(bi)] < hthr[size_t(bi)]) && hb2[size_t(bi)] > 0.0) all_ok = false;
    }
    // CH from F_I . chi_J.
    DBuf<double> pfx(size_t(B) * 6 * P), fx(size_t(B) * 6);
    {
      const dim3 g(static_cast<unsigned>(P), static_cast<unsigned>(B), 6u);
      k_b_fx<<<g, kT, 0, s>>>(F.p, X.p, nd, nrhs, pfx.p);
      TG_LAUNCH_CHECK();
      k_bsum<<<(B * 6 * 32 + 255) / 256, 256, 0, s>>>(pfx.p, P, B * 6, fx.p, nullptr, nullptr);
      TG_LAUNCH_CHECK();
    }
    std::vector<double> hfx(static_cast<size_t>(B) * 6);
    TG_CUDA(cudaMemcpyAsync(hfx.data(), fx.p, sizeof(double) * B * 6, cudaMemcpyDeviceToHost, s));
    TG_CUDA(cudaStreamSynchronize(s));
    inf.t_solve_ms = now_ms() - ts;
    inf.systems = B;
    inf.iterations_max = bt.iterations_max;
    inf.iterations_total = bt.iterations_total;
    inf.converged = all_ok ? 1 : 0;
    const double vol = double(np) * spacing * spacing * spacing;
    for (int c = 0; c < ncell; ++c) {
      double* ch = ch_out + int64_t(c) * 36;
      std::fill(ch, ch + 36, 0.0);
      for (int q = 0; q < nrhs; ++q) {
        const int J = jl[size_t(q)], bi = c * nrhs + q;
        for (int I = 0; I < 6; ++I)
          ch[I * 6 + J] =
              (double(nsolid[size_t(c)]) * c0[I][J] - hfx[size_t(bi) * 6 + I]) / vol;
      }
    }
  } catch (const Error& e) {
    set_last_error(e.what());
    rc = e.code;
  } catch (const std::bad_alloc&) {
    set_last_error("host allocation failed");
    rc = TG_ENOMEM;
  }
  inf.t_total_ms = now_ms() - t0;
  if (info) *info = inf;
  if (rc == TG_OK && !inf.converged) {
    set_last_error("homogenize: CG did not reach the requested tolerance for every system");
    rc = TG_ENONCONV;
  }
  return rc;
}
