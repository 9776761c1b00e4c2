// tg_internal.h -- shared declarations of the GB300 voxel-SIMP library.
//
// Layout in HBM (all arrays dense, structure-of-arrays where it matters):
//   element arrays  [nv]          voxel order (k*ny + j)*nx + i
//   DOF vectors     [ndof]        node-major interleaved, 3*node + comp
//   kept mask       [ndof] uint8  1 on surviving free DOFs
// Vectors of the reduced system are kept full length with zeros on non-kept
// DOFs, so the fine operator never scatters or gathers through an index list.
#pragma once

#include <cuda_runtime.h>

#include "tg_df.h"

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/topopt_gb300.h"

namespace tg {

struct Error : std::runtime_error {
  int code;
  double residual = 0.0;
  int iterations = 0;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

[[noreturn]] void raise(int code, const std::string& msg);
void set_last_error(const std::string& msg);
int device_ordinal();  // the device tg_set_device selected (0 by default)
void cuda_fail(cudaError_t e, const char* what, const char* file, int line);

#define TG_CUDA(call)                                                  \
  do {                                                                 \
    cudaError_t tg_e_ = (call);                                        \
    if (tg_e_ != cudaSuccess) ::tg::cuda_fail(tg_e_, #call, __FILE__, __LINE__); \
  } while (0)
void note_launch();
int64_t kernel_launch_count();            // launches noted by the calling thread
void add_kernel_launches(int64_t delta);  // graph replays / captures
#define TG_LAUNCH_CHECK()          \
  do {                             \
    ::tg::note_launch();           \
    TG_CUDA(cudaGetLastError());   \
  } while (0)

// Stream-ordered allocation scope.  While an AllocScope is alive on a thread,
// DBuf allocates with cudaMallocAsync on its stream and later frees with
// cudaFreeAsync on the same stream; outside any scope it uses cudaMalloc /
// cudaFree.  cudaMalloc and cudaFree are device-wide serialisation points
// (cudaFree waits for every stream), so resident jobs that come and go while
// others run -- the serving loop -- allocate stream-ordered from the device's
// memory pool instead.  A scope's stream must outlive every buffer allocated in
// it.
cudaStream_t alloc_stream();
struct AllocScope {
  cudaStream_t prev;
  explicit AllocScope(cudaStream_t s);
  ~AllocScope();
  AllocScope(const AllocScope&) = delete;
  AllocScope& operator=(const AllocScope&) = delete;
};

// Pinned host scalars from a process-wide pool (page-locked allocation is also
// a device-wide serialisation point, so it happens once per slab, not per job).
void* pinned_scalars(size_t bytes);  // bytes <= 256
void pinned_release(void* p);

// Owning device buffer.
template <class T>
struct DBuf {
  T* p = nullptr;
  size_t n = 0;
  cudaStream_t s = nullptr;  // non-null: stream-ordered allocation on s
  DBuf() = default;
  explicit DBuf(size_t count) { alloc(count); }
  DBuf(const DBuf&) = delete;
  DBuf& operator=(const DBuf&) = delete;
  DBuf(DBuf&& o) noexcept : p(o.p), n(o.n), s(o.s) { o.p = nullptr; o.n = 0; o.s = nullptr; }
  DBuf& operator=(DBuf&& o) noexcept {
    if (this != &o) {
      release();
      p = o.p; n = o.n; s = o.s;
      o.p = nullptr; o.n = 0; o.s = nullptr;
    }
    return *this;
  }
  ~DBuf() { release(); }
  void alloc(size_t count) {
    release();
    if (count) {
      const cudaStream_t as = alloc_stream();
      void* q = nullptr;
      cudaError_t e = as ? cudaMallocAsync(&q, count * sizeof(T), as)
                         : cudaMalloc(&q, count * sizeof(T));
      if (e != cudaSuccess) {
        p = nullptr;
        raise(TG_ENOMEM, "device allocation of " + std::to_string(count * sizeof(T)) +
                             " bytes failed: " + cudaGetErrorString(e));
      }
      p = static_cast<T*>(q);
      s = as;
    }
    n = count;
  }
  void release() {
    if (p) {
      if (s)
        cudaFreeAsync(p, s);
      else
        cudaFree(p);
    }
    p = nullptr;
    n = 0;
    s = nullptr;
  }
  size_t bytes() const { return n * sizeof(T); }
};

struct Grid {
  int nx = 0, ny = 0, nz = 0;
  double h = 1.0;
  int nnx = 0, nny = 0, nnz = 0;
  int64_t nv = 0, nnodes = 0, ndof = 0;
  static Grid make(int nx, int ny, int nz, double h) {
    Grid g;
    g.nx = nx; g.ny = ny; g.nz = nz; g.h = h;
    g.nnx = nx + 1; g.nny = ny + 1; g.nnz = nz + 1;
    g.nv = int64_t(nx) * ny * nz;
    g.nnodes = int64_t(g.nnx) * g.nny * g.nnz;
    g.ndof = 3 * g.nnodes;
    return g;
  }
};

// Per-class constants of the Walsh-modal hex8 operator for unit modulus:
// L[k] = lambda*h/(16*3^k), M[k] = mu*h/(16*3^k), k = number of axes a mode's
// gradient coefficient is constant along (see k_operator.cu).
struct ModalConsts {
  double L[3], M[3];
  double kdiag;  // the (common) diagonal entry of the unit-modulus Ke
  static ModalConsts make(double nu, double h);
};

// ---------------------------------------------------------------- operator
enum ApplyMode { kApply = 0, kResidual = 1, kSmooth = 2, kCheb = 3 };

// kResidual of the FP64 operator evaluated in double-float arithmetic (FP32
// pairs, ~48 significant bits): the refinement residual of the mixed form.
void launch_fine_residual_df(const Grid& g, const ModalConsts& c, const double* ef,
                             const uint8_t* kept, const double* x, const double* b, double* y,
                             cudaStream_t s);
// Fine operator on the full grid, element factors `ef` (0 = no element):
//   kApply:    y = M A x                 (M = kept mask; dot = sum x.y if dot_part)
//   kResidual: y = M (b - A x)
//   kSmooth:   y = x + omega*invdiag*(b - A x)   (invdiag is 0 off the kept set)
//   kept_node (optional): the kept mask as 3 bits per node, read by the FP32
//   column schedule instead of kept (one byte per node instead of three).
//   kSmooth with dot_part (FP32 only): partials of b . y as well.
template <class T>
void launch_fine_op(int mode, const Grid& g, const ModalConsts& mc, const T* ef,
                    const uint8_t* kept, const T* x, const T* b, const T* invdiag, T omega,
                    T* y, double* dot_part, int* nblocks_out, cudaStream_t s,
                    const uint8_t* kept_node = nullptr);
int fine_op_blocks(const Grid& g, bool fp64);  // upper bound of the partials any schedule writes

// How the FP32 fine operator is scheduled on a grid (k_operator.cu): the
// pencil kernel (the FP64 form's schedule) or the column-blocked kernel with
// one of fine_schedule_shapes() tile shapes and kz element layers per CTA.
struct FineSchedule {
  enum { kPencil = 0, kColumn = 1 };
  int kind = kColumn, shape = 0, kz = 32;
};
FineSchedule default_fine_schedule(const Grid& g);
int fine_schedule_shapes();
bool fine_schedule_valid(const FineSchedule& s);
// The schedule the FP32 operator uses on g: a process-wide override when one is
// set, else the table entry for g's dimensions (tune.cu), else the default.
FineSchedule fine_schedule_for(const Grid& g, int mode = kApply);
void set_fine_schedule_override(const FineSchedule* s);  // null clears
bool fine_schedule_known(const Grid& g);  // in the table, or an override is set
// The FP32 operator under an explicit schedule.
void launch_fine_op_sched(const FineSchedule& fs, int mode, const Grid& g, const ModalConsts& c,
                          const float* ef, const uint8_t* kept, const float* x, const float* b,
                          const float* invdiag, float omega, float* y, double* dot_part,
                          int* nblocks_out, cudaStream_t s, const uint8_t* kn);
// Times every candidate schedule of the FP32 operator on the given buffers
// (CUDA events on s) for the apply and, with b and invdiag, the residual and
// smoothing modes; publishes the fastest per mode in the table for g (one sweep
// at a time; a grid already in the table is not measured again) and returns
// the apply's.
FineSchedule autotune_fine_schedule(const Grid& g, const ModalConsts& mc, const float* ef,
                                    const uint8_t* kept, const uint8_t* kn, const float* x,
                                    float* y, double* part, cudaStream_t s,
                                    const float* b = nullptr, const float* invdiag = nullptr,
                                    int reps = 3);
// Whether the mixed form's V-cycle applies its level-1 operator on the tensor
// cores (k_coarse_tc.cu) instead of the assembled FP32 stencil; on by default.
bool level1_tc_enabled();
void set_level1_tc(bool on);
// Whether the hierarchy build forms level 1's fast-path Galerkin matrices with
// the bandwidth-bound kernel (bit-identical to the general one); on by default.
bool level1_galerkin_fast_enabled();
void set_level1_galerkin_fast(bool on);
// Whether the mixed form's V-cycle runs its small levels (from the first one of
// at most kFusedMaxNodes nodes to the coarsest) as one cluster launch
// (k_multigrid.cu) instead of a launch per step; off by default.
bool coarse_fused_enabled();
void set_coarse_fused(bool on);
// Batched apply on the periodic nx*ny*nz torus (nodes = elements per axis); see
// k_operator.cu.
template <class T>
int periodic_op_blocks(int nx, int ny, int nz);
template <class T>
void launch_periodic_op(int mode, int nx, int ny, int nz, const ModalConsts& c, const T* ef,
                        const uint8_t* kept, const T* x, const T* b, const T* invdiag, T omega,
                        T* y, double* dot_part, int nsys, int nrhs, cudaStream_t s);

// Jacobi diagonal of the fine operator: diag = kdiag * sum of adjacent factors.
void launch_fine_invdiag(const Grid& g, double kdiag, const double* ef, const uint8_t* kept,
                         double* invdiag, cudaStream_t s);

// ------------------------------------------------------------------ vectors
// Deterministic reductions: a fixed grid of kRedBlocks blocks writes partials,
// one block sums them in order.
constexpr int kRedBlocks = 608;  // 4 x 152 SMs
void launch_dot(const double* a, const double* b, int64_t n, double* part, double* out,
                cudaStream_t s);
void launch_dot_f(const float* a, const float* b, int64_t n, double* part, double* out,
                  cudaStream_t s);
void launch_sum_partials(const double* part, int n, double* out, cudaStream_t s);
// Partials of a . b (FP32 vectors) over kRedBlocks blocks, not yet summed.
void launch_dot_partials_f(const float* a, const float* b, int64_t n, double* part,
                           cudaStream_t s);
// PCG pieces with scalars living in device memory (no host round trip).
template <class T>
void launch_cg_update_xr(T* x, T* r, const T* p, const T* ap, const double* rz,
                         const double* pap, int64_t n, double* rr_part, cudaStream_t s);
// The FP32 PCG update in two kernels (alpha = rz / pAp as launch_cg_update_xr
// forms it, 0 on a breakdown): r -= alpha Ap with partials of r.r, and
// x += alpha p.
// With x0 set, launch_cg_update_r_f also writes x0 = omega invdiag .* r.
void launch_cg_update_r_f(float* r, const float* ap, const double* rz, const double* pap,
                          int64_t n, double* rr_part, cudaStream_t s,
                          const float* invdiag = nullptr, float omega = 0.0f,
                          float* x0 = nullptr);
void launch_cg_update_x_f(float* x, const float* p, const double* rz, const double* pap,
                          int64_t n, cudaStream_t s);
void launch_scale_mask(double* z, const double* r, const double* invdiag, int64_t n,
                       double* rz_part, cudaStream_t s);
template <class T>
void launch_cg_update_p(T* p, const T* z, const double* rz_new, const double* rz_old, int64_t n,
                        cudaStream_t s);
void launch_scale_d2f(float* dst, const double* src, const double* nrm2, int64_t n,
                      cudaStream_t s);
void launch_axpy_scaled_f2d(double* y, const float* x, const double* nrm2, int64_t n,
                            cudaStream_t s);
template <class T>
void launch_fill(T* a, T v, int64_t n, cudaStream_t s);
void launch_copy_d2f(float* dst, const double* src, int64_t n, cudaStream_t s);
void launch_axpy_f2d(double* y, const float* x, int64_t n, cudaStream_t s);
void launch_sub_mask(double* r, const double* b, const double* ax, const uint8_t* kept, int64_t n,
                     cudaStream_t s);
// u = kept ? x : alt; a null x or alt reads as zeros.
void launch_mask_select(double* u, const double* x, const double* alt, const uint8_t* kept,
                        int64_t n, cudaStream_t s);

// ---------------------------------------------------------------- SIMP
void launch_modulus(const double* rho, const uint8_t* elem, int64_t n, double E0, double p,
                    double rho_min, int law, double emin, double* E, cudaStream_t s);
// Compliance + sensitivity sweep: dc[e], and per-block partial compliances.
void launch_sensitivity(const Grid& g, const ModalConsts& mc, const double* rho,
                        const uint8_t* elem, const double* u, double E0, double p,
                        double rho_min, int law, double emin, double* dc, double* c_part,
                        int* nparts, cudaStream_t s,
                        bool double_float = false);

struct FilterStencil {
  int R = 0, n = 0;
  std::vector<int> di, dj, dk;
  std::vector<double> w;
  static FilterStencil make(double radius);
};
// Uploads the stencil into `buf`; returns the device pointer kernels take.
void* filter_stencil_device(const FilterStencil& st, DBuf<unsigned char>& buf, cudaStream_t s);
void launch_weight_sum(const Grid& g, const void* st, int ns, const uint8_t* act, double* hs,
                       cudaStream_t s);
void launch_filter_fwd(const Grid& g, const void* st, int ns, const uint8_t* act,
                       const double* hs, const double* x, double* out, cudaStream_t s);
void launch_filter_adj(const Grid& g, const void* st, int ns, const uint8_t* act,
                       const double* hs, const double* s_in, double* tmp, double* out,
                       cudaStream_t s);
// Up to kOcMulti bisection candidates (c = 1/sqrt(lambda)) evaluated in one pass.
constexpr int kOcMulti = 16;
struct OcCands {
  int k;
  double c[kOcMulti];
};
// The same candidates as double-float pairs (tg_df.h) for the device.
struct OcCandsDF {
  int k;
  df c[kOcMulti];
};
// out[k] = sum_e dv_e clamp(sq_e c_k, lo_e, hi_e) in double-float arithmetic;
// sq, lo, hi, dvd are the double-float fields launch_oc_prepare writes (8 bytes
// per voxel each, in double-sized buffers); part holds k * kRedBlocks partials.
void launch_oc_volume_multi(const double* sq, const double* lo, const double* hi,
                            const double* dvd, int64_t n, const OcCands& cs, double* part,
                            double* out, cudaStream_t s);
void launch_oc_candidate(const double* x, const double* dcf, const double* dvf,
                         const uint8_t* act, int64_t n, double lambda, double move,
                         double rho_min, bool carry, double* xnew, cudaStream_t s);
// Heaviside projection (simp.cpp:352-365): out = projected xt on the design
// voxels (act; every voxel when act is null), xt elsewhere; deriv (optional)
// the derivative there, 0 elsewhere.  Either output may be null.
void launch_project(const double* xt, const uint8_t* act, int64_t n, double beta, double eta,
                    double* out, double* deriv, cudaStream_t s);
// dproj = derivative(xtilde), dcp = dc * dproj on the design voxels, 0 elsewhere.
void launch_proj_chain(const double* xtilde, const double* dc, const uint8_t* act, int64_t n,
                       double beta, double eta, double* dproj, double* dcp, cudaStream_t s);
// Projected OC candidates for ls.k multipliers; candidate j at cand + j * n.
struct ProjLambdas {
  int k;
  double lam[kOcMulti];
};
void launch_oc_candidates_projected(const double* x, const double* dcf, const double* dvf,
                                    const uint8_t* act, int64_t n, const ProjLambdas& ls,
                                    double move, double rho_min, bool carry, double* cand,
                                    cudaStream_t s);
// out[j] = sum over design voxels of heaviside_project(filter(cand_j)), j < k;
// part holds k * kRedBlocks partials.
void launch_proj_volume(const Grid& g, const void* st, int ns, const uint8_t* act,
                        const double* hs, const double* cand, int k, double beta, double eta,
                        double* part, double* out, cudaStream_t s);
// MMA (mma_joint.cpp): the per-voxel fields of one run's subproblem.
struct MmaFields {
  double *low, *upp, *xold1, *xold2, *p0, *q0, *p1, *q1, *al, *be;
};
// Asymptotes, coefficients and move box from x, dcf (unscaled), dvf; tsum[0] =
// sum over the design set of p1/(U - x) + q1/(x - L).  scale_bits: 1 scratch word.
void launch_mma_prepare(const MmaFields& m, const double* x, const double* dcf, const double* dvf,
                        const uint8_t* act, int64_t n, int iter, double move, double xmin,
                        uint64_t* scale_bits, double* part, double* tsum, cudaStream_t s);
// out[j] = the dual's constraint sum at ls.lam[j], j < ls.k.
void launch_mma_dual(const MmaFields& m, const uint8_t* act, int64_t n, const ProjLambdas& ls,
                     double* part, double* out, cudaStream_t s);
// x_new(lambda) on the design set, 0 elsewhere.
void launch_mma_candidate(const MmaFields& m, const uint8_t* act, int64_t n, double lam,
                          double* xnew, cudaStream_t s);
// hex8_stress at every voxel centre where solid[e] and (rho null or rho[e] >
// iso): von Mises and the 6 stresses (either output may be null; 0 elsewhere),
// and into peaks[0..2] (zeroed by the caller) the bit patterns of the peak von
// Mises and interlayer tension along bdir, and the printed-voxel count.
void launch_element_stress(const Grid& g, const uint8_t* solid, const double* rho,
                           const double* u, double E, double nu, double h, const double* bdir,
                           double iso, double* vm_out, double* sig_out, uint64_t* peaks,
                           cudaStream_t s);
// FrozenSolid (1) -> 1, FrozenVoid (2) -> 0 on the physical density.
void launch_mask_pins(const uint8_t* eff, int64_t n, double* xphys, cudaStream_t s);
// Active domain (k_active.cu): the mask into `out` (tmp: nv scratch bytes) and
// its count of ones; the escape count of rho against prev.  Counts are reset
// on the stream first.
void launch_active_domain_mask(int nx, int ny, int nz, const uint8_t* tags, const double* rho,
                               double density_min, int band, uint8_t* out, uint8_t* tmp,
                               unsigned long long* count, cudaStream_t s);
void launch_active_domain_escape(const uint8_t* tags, const double* rho, const uint8_t* prev,
                                 double density_min, int64_t nv, unsigned long long* count,
                                 cudaStream_t s);
// Exact (fixed-point, order independent) sum of a non-negative field over the
// solid voxels; returns per-block 192-bit partials, then the final total.
int exact_sum_blocks();
// sq = x sqrt(B), lo, hi (the move window) and dvd = dvf, as double-float pairs.
void launch_oc_prepare(const double* x, const double* dcf, const double* dvf, const uint8_t* act,
                       int64_t n, double move, double rho_min, double* sq, double* lo, double* hi,
                       double* dvd, cudaStream_t s);
void launch_exact_sum(const double* v, const uint8_t* act, int64_t n, uint64_t* part,
                      uint64_t* total, int* inexact, cudaStream_t s);
double fma_probe_tflops(bool fp64);
void launch_absdiff_max(const double* a, const double* b, int64_t n, double* part, double* out,
                        cudaStream_t s);

}  // namespace tg
