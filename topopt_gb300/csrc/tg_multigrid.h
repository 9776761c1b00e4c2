// tg_multigrid.h -- launchers of the multigrid kernels (k_multigrid.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

namespace tg {

// Entries per node of a stored coarse stencil: the self block and the 13 forward
// neighbour blocks, 3x3 each (the backward blocks are their transposes).
constexpr int kStencilEntries = 14 * 9;

// Element and node extents of one hierarchy level.  align (coarse levels): how
// an odd finer axis (2m+1 elements) is coarsened.  0 -- the reference's
// index-space padding: coarse node m+1 would coincide with fine node 2m+2,
// beyond the grid, so it is inactive and the last fine node interpolates half
// of coarse node m only (multigrid.cpp:391-459).  1 -- boundary-aligned: coarse
// node m+1 coincides with the last fine node 2m+1 (prolongation weight 1) and
// the last coarse element spans a single fine element, so the coarse space keeps
// the rigid and smooth modes up to the boundary.
struct MgDims {
  int ex, ey, ez, nnx, nny, nnz;
  int align = 0;
};

// spos (FP32, optional): per coarse element, < 0 on the fast path (sum_c f_c G_c;
// the level-1 tensor-core operator's special-element positions), where a
// bandwidth-bound kernel forms the matrix.
template <class T>
void mg_galerkin_level1(const MgDims& fd, const MgDims& cd, const T* ef, const uint8_t* fact,
                        const uint8_t* cact, const T* Ke, const T* G, T* Kc, cudaStream_t s,
                        const int* spos = nullptr);
template <class T>
void mg_galerkin_coarse(const MgDims& fd, const MgDims& cd, const T* Kf, const uint8_t* cact,
                        T* Kc, cudaStream_t s);
template <class T>
void mg_assemble_stencil(const MgDims& d, const T* Kel, const uint8_t* act, T* A, T* invdiag,
                         cudaStream_t s);
void mg_to_float(const double* src, float* dst, int64_t n, cudaStream_t s);
// One Chebyshev smoothing step (kCheb): the direction vector it updates in
// place (the level's precision), the level's coefficient table (mg_cheb_table)
// and the step index within the polynomial.
struct ChebStep {
  void* dir_ = nullptr;
  const float* coef = nullptr;
  int step = 0;
};
// Chebyshev coefficients of steps 0 .. m-1 on [lam/ratio, lam] (lam = *lam on
// the device) into coef[0 .. 2m): coef[0] = 1/theta, coef[2k], coef[2k+1] =
// rho_k rho_{k-1}, 2 rho_k / delta for k >= 1, each rounded to FP32 once.
// Computed once per hierarchy build: the smoothing kernels read them instead of
// evaluating the FP64 recurrence in every thread (GB300's FP64 rate is 1/64 of
// its FP32 rate).
constexpr int kChebCoefStride = 16;  // up to 8 steps
void mg_cheb_table(const double* lam, double ratio, int m, float* coef, cudaStream_t s);
template <class T>
void mg_stencil_op(int mode, const MgDims& d, const T* A, const uint8_t* act, const T* x,
                   const T* b, const T* invdiag, T omega, T* y, cudaStream_t s,
                   ChebStep ch = ChebStep{});
// lambda_max(D^-1 A) of a stencil level by `iters` power-iteration steps (v, w:
// level-sized scratch), times `safety`, into lam[0] on the device.
template <class T>
void mg_lambda_max(const MgDims& d, const T* A, const uint8_t* act, const T* invdiag, T* v,
                   T* w, int iters, double safety, double* part, double* nrm2, double* lam,
                   cudaStream_t s);
template <class T>
void mg_jacobi_first(const T* b, const T* invdiag, T omega, int64_t n, T* x, cudaStream_t s);
// The coarse level's first smoothing step from a zero iterate, taken by the
// restriction that forms its right-hand side (it needs no operator): kind 1
// damped Jacobi, x = omega dinv b (as mg_jacobi_first); kind 2 Chebyshev step 0,
// chd = coef[0] dinv b and x = 0 + chd (as the kCheb stencil step on x = 0).
template <class T>
struct FirstStep {
  int kind = 0;  // 0: none
  const T* dinv = nullptr;
  T omega = T(0);
  const float* coef = nullptr;
  T* x = nullptr;
  T* chd = nullptr;
};
template <class T>
void mg_restrict(const MgDims& fd, const MgDims& cd, const T* rf, const uint8_t* cact, T* bc,
                 cudaStream_t s, FirstStep<T> first = FirstStep<T>{});
template <class T>
void mg_prolong_add(const MgDims& fd, const MgDims& cd, const T* ec, const uint8_t* fact, T* xf,
                    cudaStream_t s);
template <class T>
void mg_dense_from_stencil(const MgDims& d, const T* A, const int* cidx, int nc, double* D,
                           cudaStream_t s);
void mg_cholesky(double* D, int nc, int* fail, cudaStream_t s);
// Explicit inverse of the coarsest operator from its factor (small levels).
void mg_chol_inverse(const double* L, int nc, double* Li, double* Ainv, cudaStream_t s);
// x = Ainv b over the compact numbering (cidx: dof -> compact, cdof: compact -> dof).
template <class T>
void mg_coarse_inv_apply(const double* Ainv, int nc, const int* cidx, const int* cdof,
                         int64_t ndof, const T* b, T* x, cudaStream_t s);
template <class T>
void mg_chol_solve(const double* L, int nc, const int* cidx, int64_t ndof, const T* b, T* x,
                   double* work, cudaStream_t s);

// The small levels of the FP32 V-cycle in one launch of one thread-block cluster
// (k_multigrid.cu).  L[0] is the first fused level (its right-hand side b set by
// the finer level's restriction), L[nlev-1] the coarsest (solved with the dense
// inverse Ainv over the compact numbering cidx/cdof).  Each smoothed level has
// two iterate buffers: xp (the iterate on entry, as the launch-by-launch
// V-cycle's X) and xq; smoothing is Chebyshev of degree cheb_m (> 0, direction
// chd, coefficient table coef on the device) or damped Jacobi with `sweeps` sweeps per
// side.  The fused part starts at the first level with at most kFusedMaxNodes
// nodes: a cluster of kFusedThreads-thread CTAs covers a few DOFs per thread.
constexpr int kFusedMaxLevels = 12;
constexpr int64_t kFusedMaxNodes = 4096;
constexpr int kFusedThreads = 512;
struct FusedLevel {
  MgDims d;
  const float* A = nullptr;
  const uint8_t* act = nullptr;
  const float* dinv = nullptr;
  float* xp = nullptr;
  float* xq = nullptr;
  float* b = nullptr;
  float* chd = nullptr;
  const float* coef = nullptr;  // Chebyshev coefficients (mg_cheb_table)
};
struct FusedCoarse {
  int nlev = 0;
  FusedLevel L[kFusedMaxLevels];
  int cheb_m = 0, sweeps = 1;
  float omega = 0.6f;
  const double* Ainv = nullptr;
  int nc = 0;
  const int* cidx = nullptr;
  const int* cdof = nullptr;
};
// CTAs in the fused launch's cluster (16 where the device co-schedules that
// many, else 8, 4, 2, 1).
int fused_coarse_blocks();
void mg_coarse_vcycle_fused(const FusedCoarse& fc, cudaStream_t s);

// The FP32 level-1 Galerkin operator on the tensor cores (k_coarse_tc.cu):
// y = A1 x (kApply), b - A1 x (kResidual) or x + omega D^-1 (b - A1 x) (kSmooth),
// masked by act, from the fine FP32 factors ef and the 8 child blocks G (FP32,
// [8][576] corner-bit order).  The nspec coarse elements off the fast path
// (slist; spos[ce] = position in slist or -1) are applied from their stored
// matrices Kel by a pre-pass into yspec (nspec x 24).  A wait that runs out
// sets *err.
void mg_level1_tc(int mode, const MgDims& fd, const MgDims& cd, const float* ef,
                  const uint8_t* act, const int* spos, const int* slist, int nspec,
                  const float* Kel, const float* G, const float* x, const float* b,
                  const float* invdiag, float omega, float* y, float* yspec, int* err,
                  cudaStream_t s);

}  // namespace tg
