// tg_solver.h -- the reduced FEA system and its solvers (host orchestration).
#pragma once

#include <memory>
#include <vector>

#include "tg_internal.h"
#include "tg_multigrid.h"

namespace tg {

// Host Ke of the reference's 2x2x2 Gauss integration (hex_element.cpp:23-115),
// row-major 24x24 in the reference's local node order.
void hex8_ke(double E, double nu, double h, double* ke576);

// The design-independent part of the reduced, void-gated system
// (matfree.cpp:670-834): which elements exist, which DOFs survive, the load
// vector and the prescribed field.  Built once per grid + BCs + active mask.
struct FineProblem {
  Grid g;
  double nu = 0.3;
  ModalConsts mc{};
  std::vector<double> ke;          // unit-modulus Ke, reference order
  std::vector<uint8_t> elem_h;     // element exists (solid and active) [nv]
  std::vector<uint8_t> kept_h;     // [ndof]
  std::vector<uint8_t> kept_node_h;  // [nnodes] kept bits per node (bit k: DOF 3n+k)
  std::vector<double> f_h;         // load vector [ndof]
  std::vector<double> up_h;        // prescribed field [ndof]
  std::vector<uint8_t> fixed_h;    // Dirichlet mask [ndof]
  bool nonzero_bc = false;
  int64_t ng = 0, n_free = 0;
  DBuf<uint8_t> elem, kept, kept_node;
  DBuf<double> f, up;

  // Throws Error(TG_EINVAL) on bad indices, Error(TG_ESINGULAR) on a void-only
  // system or a load on a void DOF (the load check uses f; with non-zero
  // prescribed values the caller re-checks with f - K u_p).
  void build(const tg_grid& grid, double poisson, const tg_dirichlet_bc* bcs, int nbc,
             const tg_nodal_load* loads, int nloads, const uint8_t* active_mask,
             cudaStream_t s);
  size_t device_bytes() const;
};

struct SolverStats {
  int iterations = 0;
  double residual = 0.0;
  bool converged = false, used_mg = false, hier_built = false;
  int mg_levels = 0, mg_cycles = 0, refinements = 0;
  bool mixed_fallback = false;
  int inner_breakdowns = 0;
  int64_t matvecs = 0, matvecs_lowp = 0;
  double t_mg_build_ms = 0.0, t_solve_ms = 0.0;
};

// The solver holds device state sized for one FineProblem; per solve it takes
// element factors E (device, [nv], 0 = no element) and returns x on the kept
// DOFs (full length, 0 elsewhere).
class Solver {
 public:
  Solver(const FineProblem& fp, const tg_solve_options& opt, cudaStream_t s);
  ~Solver();
  // Set the element factors for the next solve: rebuilds the Jacobi diagonal,
  // the reduced right-hand side and (MG) the numeric hierarchy.
  void set_modulus(const double* E);
  // Solve A x = rhs to ||r|| <= tol ||rhs||.  guess (device, ndof) may be null.
  // Writes the full displacement u = x on kept DOFs, u_p elsewhere.
  SolverStats solve(double tol, int max_it, const double* guess, double* u);
  // y = A x on the full grid (no mask), for the public apply entry point.
  void apply_unmasked(const double* E, const double* x, double* y);
  const double* rhs() const { return rhs_.p; }
  // Time `reps` fine-operator launches (FP64 or FP32) on the current factors.
  // form: 0 FP64, 1 FP32, 2 the double-float residual kernel.
  double time_operator(int form, int reps);
  // Level 1 of the FP32 V-cycle applied to a seeded vector by the assembled
  // stencil and by the tensor-core operator: max |difference| / max |stencil|.
  double check_level1();
  size_t device_bytes() const;
  int levels() const { return int(levels_.size()) + 1; }

 private:
  struct Level;
  struct Impl;
  void build_structure();
  template <class T>
  bool build_numeric();

  bool mgpcg(double tol, int max_it, bool warm, SolverStats& st);
  bool jacobi_pcg(double tol, int max_it, bool warm, SolverStats& st);
  bool mixed_refine(double tol, int max_it, bool warm, SolverStats& st);
  template <class T>
  T* vcycle(const T* b, double* bz = nullptr, bool x0_ready = false);
  template <class T>
  T* vcycle_level(size_t l, bool first_done = false);  // returns the level's result buffer
  template <class T>
  FirstStep<T> first_step(size_t l);  // level l's first sweep, for the restriction into it
  float* fused_coarse_vcycle();
  template <class T>
  bool inner_pcg(int max_it, double rel_tol, SolverStats& st, int* iters);
  bool build_inner_graph();
  double read_scalar(int idx);
  void read_scalars(int idx0, int n, double* out);

  const FineProblem& fp_;
  tg_solve_options opt_;
  cudaStream_t s_;
  double omega_ = 0.6;
  int budget_ = 300;
  int sweeps_ = 1;  // damped-Jacobi sweeps per side of the coarse correction
  bool df_residual_ = true;  // mixed: refinement residual in double-float arithmetic
  bool mixed_partial_ = false;  // the last mixed attempt ran out of budget with progress
  // Chebyshev smoothing of the FP32 V-cycle's levels >= 2: polynomial degree
  // (0 = damped Jacobi), interval [lmax / ratio, lmax] of D^-1 A, lmax from a
  // power iteration times a safety factor, per hierarchy build.
  int cheb_m_ = 0;
  double cheb_ratio_ = 30.0;
  int cheb_iters_ = 10;
  double cheb_safety_ = 1.1;
  DBuf<double> lam_;     // lambda_max per level
  DBuf<double> pipart_;  // per level: the power iteration's partials and norm
  std::vector<cudaStream_t> pi_streams_;  // per level, the power iterations' streams
  std::vector<cudaEvent_t> pi_events_;
  cudaEvent_t pi_fork_ = nullptr;
  void ensure_pi_streams(size_t nlev);
  DBuf<float> chc_;        // Chebyshev coefficients per level (kChebCoefStride each)
  void refinement_residual();  // r = b - A x (FP64 in, FP64 out) for the mixed loop
  bool mixed_ = false;
  // fine state
  const double* E_ = nullptr;
  DBuf<double> invdiag_, rhs_, x_, r_, z_, p_, ap_, t0_, t1_;
  DBuf<float> Ef_, invdiagf_, xf_, rf_, zf_, pf_, apf_, t0f_, t1f_;
  DBuf<double> part_, scal_;
  double* h_scal_ = nullptr;  // pinned
  int part_n_ = 0;
  // hierarchy
  std::vector<std::unique_ptr<Level>> levels_;  // levels 1..L-1
  DBuf<double> keb_, G_;                         // Ke in corner-bit order, 8 G_c
  DBuf<float> kebf_, Gf_;
  bool have_mg_ = false, numeric_ok_ = false, numeric_[2] = {false, false};
  double mg_build_ms_ = 0.0;
  int64_t fine_matvecs_ = 0, lowp_matvecs_ = 0;
  int nc_ = 0;
  DBuf<int> cidx_, cdof_, chol_fail_;
  DBuf<double> chol_, chol_work_, chol_li_, chol_inv_;
  // The mixed inner PCG loop as one CUDA graph: a conditional WHILE node whose
  // body is one PCG iteration (V-cycle, update, apply) ending in a kernel that
  // decides, on the device, whether another iteration runs.
  struct InnerGraph;
  std::unique_ptr<InnerGraph> ig_;
  bool ig_failed_ = false, use_graph_ = true;
  DBuf<int> istate_;           // [0] iterations done, [1] budget, [2] breakdown
  // Level 1 of the FP32 V-cycle on the tensor cores: per coarse element, 1 when
  // its matrix is not sum_c E_c G_c (a Dirichlet or untouched fine DOF in a
  // solid child, an inactive coarse DOF or a half element) and the stored
  // matrix is applied instead; the kernel's timeout flag.
  bool l1_tc_ = false;
  int nspec1_ = 0;
  DBuf<int> spos1_, slist1_;  // per coarse element: position in slist1_ or -1
  DBuf<float> yspec1_;        // their outputs, nspec1_ x 24
  DBuf<int> tc_err_;  // a tensor-core completion wait that ran out
  // The small levels of the FP32 V-cycle in one cluster launch.
  size_t fused_level_ = 0;  // first level of the fused cluster launch (0: none)
  bool l1_stencil_ok_ = true;  // the FP32 level-1 stencil is assembled (not only its diagonal)
  void level1_stencil();
  // The FP32 PCG's deferred x += alpha p (alpha from scal_[6], scal_[7]; p in
  // pf_): pending until flush_x() runs it on s_ or fork_x() on the side stream
  // s2_ as the V-cycle enters side_level_; join_x() makes s_ wait for it.
  bool pending_x_ = false, side_joined_ = true;
  size_t side_level_ = 0;
  cudaStream_t s2_ = nullptr;
  cudaEvent_t ev_fork_ = nullptr, ev_join_ = nullptr;
  void ensure_side();
  bool fork_x();
  void join_x() noexcept;
  void flush_x();
  void level1_op(int mode, Level& L, float omega);
  int* h_ist_ = nullptr;       // pinned mirror of istate_
};

}  // namespace tg
