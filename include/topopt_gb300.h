/*
 * topopt_gb300.h -- C ABI of the GB300-native voxel-SIMP inner loop.
 *
 * A drop-in for the reference's optimizer/solver entry points (Anarkissed/TopOpt,
 * core/).  Every entry point takes caller-owned HOST buffers and sizes, copies
 * them to the device, runs hand-written sm_103a kernels and copies results back;
 * nothing throws across the ABI.  The resident-job API (tg_job_*) keeps a design's
 * density, displacement and multigrid hierarchy on the device across design
 * iterations.
 *
 * Conventions are the reference's (core/include/topopt/fea.hpp:18-29, :140-171):
 *   voxel (i,j,k) -> (k*ny + j)*nx + i; node (a,b,c) -> (c*(ny+1) + b)*(nx+1) + a;
 *   DOF = 3*node + component; Hex8 nodes bottom face CCW then top face CCW.
 *
 * Errors: every function returns a tg_status; tg_last_error() returns the
 * calling thread's message for the last failure.  The codes map the reference's
 * exception classes (fea.hpp:418-469, matfree.cpp:782-814):
 *   TG_EINVAL      std::invalid_argument   (sizes, indices, E <= 0, nu range)
 *   TG_ESINGULAR   std::runtime_error      (void-only system, load on a void DOF)
 *   TG_ENONCONV    SolverNonConvergence    (tg_cg_info carries iterations/residual)
 *   TG_EDEADLINE   SolverDeadlineExceeded
 *   TG_EDEVICE     a CUDA error (the message names the call)
 *   TG_ECANCELLED  the caller's cancel flag was observed
 *
 * Threading: every entry point is re-entrant; a tg_job is driven by one thread
 * at a time and owns one CUDA stream.
 */
#ifndef TOPOPT_GB300_H
#define TOPOPT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  TG_OK = 0,
  TG_EINVAL = 1,
  TG_ESINGULAR = 2,
  TG_ENONCONV = 3,
  TG_EDEADLINE = 4,
  TG_EDEVICE = 5,
  TG_ENOMEM = 6,
  TG_ECANCELLED = 7
} tg_status;

/* VoxelGrid (core/include/topopt/voxel.hpp:56-92).  `tags` holds one VoxelTag
 * byte per voxel (0 = Empty, anything else solid); NULL means every voxel is
 * Interior. */
typedef struct {
  int32_t nx, ny, nz;
  double spacing;
  const uint8_t* tags;
} tg_grid;

/* DirichletBC / NodalLoad (core/include/topopt/fea.hpp:173-187). */
typedef struct {
  int32_t node, component;
  double value;
} tg_dirichlet_bc;
typedef struct {
  int32_t node, component;
  double value;
} tg_nodal_load;

/* SimpParams (core/include/topopt/simp.hpp:36-40).  material_law 0 is the
 * reference law E = clamp(rho, rho_min, 1)^p * E0 (simp.cpp:44-47, :656);
 * 1 is the modified law E = Emin + rho^p (E0 - Emin) with Emin = e_min. */
typedef struct {
  double youngs_modulus, poisson, penalty, density_min;
  int32_t material_law;
  double e_min;
} tg_simp_params;

typedef enum { TG_SOLVER_MGCG = 0, TG_SOLVER_JACOBI_CG = 1 } tg_solver_kind;
typedef enum { TG_PREC_FP64 = 0, TG_PREC_MIXED = 1 } tg_precision;
/* tg_matfree_apply only: the FP64 operator evaluated in double-float arithmetic
 * (the mixed form's refinement residual kernel). */
enum { TG_APPLY_DF = 2 };
/* tg_job_time_operator only: the level-1 operator of the mixed form's V-cycle,
 * residual mode -- the assembled FP32 stencil or the tensor-core operator. */
enum { TG_APPLY_L1_STENCIL = 3, TG_APPLY_L1_TC = 4 };

/* Solver knobs.  Zero-initialised means: MG-PCG, FP64, the deepest hierarchy the
 * grid allows, the reference's iteration budget of 300 MG cycles before the
 * Jacobi-PCG fallback (multigrid.cpp:122), damped Jacobi w = 0.6 with 1+1 sweeps
 * (multigrid.cpp:72-76). */
/* Multigrid coarsening of odd axes.  REFERENCE: the reference's index-space
 * padding (multigrid.cpp:391-459; the plain FP64 form's default).  ALIGNED: the
 * last coarse node sits on the last fine node (the mixed form's default):
 * the same Galerkin method with a coarse space that keeps the smooth modes at
 * odd boundaries -- far fewer iterations on odd grids, same solution. */
enum { TG_COARSEN_DEFAULT = 0, TG_COARSEN_REFERENCE = 1, TG_COARSEN_ALIGNED = 2 };
enum { TG_GRAPH_ON = 0, TG_GRAPH_OFF = 1 };

typedef struct {
  int32_t solver;          /* tg_solver_kind */
  int32_t precision;       /* tg_precision */
  int32_t mg_levels;       /* 0 = deepest (coarsest axis >= 2 elements) */
  int32_t mg_iter_budget;  /* 0 = 300 */
  double omega;            /* 0 = 0.6 */
  double inner_tolerance;  /* mixed: relative tolerance of each FP32 inner solve; 0 = 0.3x the
                              reduction still needed, within [1e-5, 0.1] */
  int32_t max_refinements; /* mixed: outer FP64 refinement steps, 0 = 20 */
  int32_t coarsening;      /* odd-axis coarsening: TG_COARSEN_* (0 = the form's default) */
  int32_t graph_mode;      /* mixed: TG_GRAPH_ON (default, 0) runs the inner PCG loop as one
                              CUDA graph with a device-side loop condition; TG_GRAPH_OFF
                              drives it from the host (same arithmetic, same results) */
  int32_t smooth_sweeps;   /* damped-Jacobi sweeps before and after the coarse correction
                              on every level (0 = 1, the reference's smoother) */
  int32_t mixed_residual;  /* mixed: how the FP64 refinement residual b - A x is evaluated:
                              TG_RESIDUAL_DF (0, default) in double-float arithmetic (FP32
                              pairs, ~48 significant bits, on the FP32 pipe), TG_RESIDUAL_FP64
                              with the native FP64 operator */
  int32_t coarse_smoother; /* mixed: the smoother of the FP32 V-cycle's levels >= 2:
                              TG_SMOOTHER_AUTO (0) Chebyshev on grids of >= 200K elements,
                              Jacobi below; TG_SMOOTHER_JACOBI (1) damped Jacobi (the
                              reference's); TG_SMOOTHER_CHEBYSHEV (2) a degree-4 Chebyshev
                              polynomial in D^-1 A on [lmax / 30, lmax], lmax by power
                              iteration per hierarchy build.  The FP64 V-cycle always uses
                              damped Jacobi. */
} tg_solve_options;

enum { TG_RESIDUAL_DF = 0, TG_RESIDUAL_FP64 = 1 };
enum { TG_SMOOTHER_AUTO = 0, TG_SMOOTHER_JACOBI = 1, TG_SMOOTHER_CHEBYSHEV = 2 };

/* CgInfo subset (core/include/topopt/fea.hpp:272-382). */
typedef struct {
  int32_t converged, iterations;
  double residual;
  int32_t used_multigrid, mg_levels, hier_built, mg_cycles_attempted;
  int64_t matvecs;        /* fine FP64 operator applies */
  int64_t matvecs_lowp;   /* fine reduced-precision operator applies */
  int32_t refinements;    /* mixed: outer FP64 refinement steps */
  int32_t ng;             /* surviving (kept) DOFs */
  int32_t mixed_fallback; /* mixed: the FP32 inner solve failed and FP64 MG-PCG took over */
  int32_t inner_breakdowns;
  double t_build_ms, t_mg_build_ms, t_solve_ms, t_total_ms;
} tg_cg_info;

/* One stage of the Heaviside beta continuation (ProjectionStage,
 * core/include/topopt/simp.hpp:519-523). */
typedef struct {
  double beta;        /* projection sharpness, finite and > 0 */
  double move;        /* OC move limit of the stage, > 0 */
  int32_t iterations; /* OC iterations of the stage, >= 1 */
} tg_projection_stage;

/* The OC subset of SimpOptions (core/include/topopt/simp.hpp:1028-1138,
 * projection and projection_eta :1426-1444).  projection NULL or
 * projection_stages 0: the unprojected loop, governed by move and
 * max_iterations.  Otherwise the stages run in order, each its own iterations
 * at its own beta and move (a stage ends early when the design change drops
 * below change_tol), the analysis density is heaviside_project(filter(x), beta,
 * projection_eta) on the design voxels and the volume constraint is on that
 * projected density; projection_eta must then be in (0, 1) (the reference's
 * default is 0.5). */
typedef struct {
  double volume_fraction, filter_radius, move, change_tol, cg_tolerance;
  int32_t max_iterations, cg_max_iterations;
  tg_solve_options solve;
  const tg_projection_stage* projection;
  int32_t projection_stages;
  double projection_eta;
  /* Warm start (SimpOptions::initial_design, simp.hpp:1557-1575): NULL is the
   * uniform start; otherwise a raw seed density per voxel whose mean over the
   * design set is rescaled to volume_fraction, clamped to [density_min, 1] and
   * filtered once (warm_start_design, simp.cpp:324-344). */
  const double* initial_design;
  /* The design updater (SimpOptions::updater, simp.hpp:1119): TG_UPDATER_OC (0,
   * the default) or TG_UPDATER_MMA (Svanberg's MMA, simp.cpp:1420-1489,
   * mma_joint.cpp; no projection plan).  MMA ends a run on the objective plateau
   * (mma_objective_plateau, simp.cpp:1081-1134) when mma_plateau_window > 0
   * (the reference's defaults are 10, 1e-3, 0.05, 3), else on change_tol. */
  int32_t updater;
  int32_t mma_plateau_window;
  double mma_plateau_tol, mma_plateau_min_drop;
  int32_t mma_plateau_flat_windows;
  /* Active domain (SimpOptions::active_domain_band, simp.hpp:1185-1227): 0 (the
   * default) off; > 0 every trajectory solve runs on the material plus a band of
   * this half-width in voxels (tg_active_domain_mask), out-of-band elements get
   * no energy and no sensitivity; < 0 the band is tg_active_domain_auto_band
   * (filter_radius).  The certification solve is always on the full domain.
   * The mask is switched off for the rest of the run (one way) on the first
   * escape, after 5 consecutive iterations at an active fraction >= 0.85, or
   * when a restricted solve fails (that iteration is then re-solved on the full
   * domain); tg_simp_result records which. */
  int32_t active_domain_band;
} tg_simp_options;

enum { TG_UPDATER_OC = 0, TG_UPDATER_MMA = 1 };

/* One row of the per-iteration record (SimpIteration + the observation fields
 * of simp.hpp:913-960 that the iterations.csv schema carries). */
typedef struct {
  int32_t iteration;
  double compliance, change, volume_fraction;
  int32_t cg_iterations, mg_levels, used_multigrid, oc_volume_evals;
  double t_filter_ms, t_solve_ms, t_sensitivity_ms, t_update_ms, t_total_ms;
  double t_device_ms; /* CUDA-event time of the iteration on the job's stream */
  int64_t fine_matvecs, fine_matvecs_lowp;
  int32_t oc_volume_passes; /* passes over the fields that evaluated the bisection's volumes */
  double beta; /* projection sharpness of this iteration's stage; 0 when unprojected */
  int32_t hier_built;          /* a multigrid hierarchy was built for this solve */
  int32_t mg_cycles_attempted; /* V-cycles this solve ran */
  int32_t oc_exact_evals;      /* bisection branches the fast volume bound could not decide */
  int32_t oc_host_fallbacks;   /* of those, decided by the host's sequential sum */
  double active_fraction;      /* active elements / solid elements of this iteration's solve;
                                  1 when it ran on the full domain */
} tg_simp_iteration;

typedef struct {
  int32_t iterations, converged, cancelled, infeasible, non_convergent;
  double compliance, initial_compliance, volume_fraction;
  /* Active domain (SimpOptimizeResult, simp.hpp:1735-1761): the band the run
   * used (0 = off), whether and at which 1-based iteration the mask was
   * switched off and why, the escapes counted when the escape latch fired, and
   * the mean of the per-iteration active fractions (1 when off). */
  int32_t active_domain_band, active_domain_latched, active_domain_latch_iteration;
  int64_t active_domain_escape_count;
  double active_fraction_mean;
  char active_domain_latch_reason[256];
} tg_simp_result;

/* Progress hook (TopOptBridge.hpp:262-263): called on the optimizing thread
 * after every design iteration. */
typedef void (*tg_progress_fn)(void* ctx, int32_t iteration, double compliance, double change);

const char* tg_last_error(void);
/* Device ordinal the library uses (set before the first call; default 0). */
int tg_set_device(int32_t device);
/* Library and kernel build identification. */
const char* tg_version(void);

/* hex8_stiffness (core/src/fea/hex_element.cpp:93-115): 24x24 row-major Ke. */
int tg_hex8_stiffness(double youngs_modulus, double poisson, double element_size,
                      double* ke576);

/* fea_matfree_apply (core/include/topopt/fea.hpp:760-766; matfree.cpp:1079-1098):
 * y = K u over the full grid.  youngs_per_voxel NULL -> uniform youngs_modulus.
 * precision TG_PREC_MIXED runs the FP32 operator (inputs rounded to float),
 * TG_APPLY_DF the double-float one. */
int tg_matfree_apply(const tg_grid* grid, double youngs_modulus, double poisson,
                     const double* youngs_per_voxel, int32_t precision, const double* u,
                     double* y);

/* mf_build_reduced's void-DOF gate (core/src/fea/matfree.cpp:670-834): kept[d] = 1
 * for surviving DOFs, rhs = f - K u_p on them, invdiag the Jacobi inverse
 * diagonal; all ndof long.  Returns TG_ESINGULAR on the reference's rejections. */
int tg_build_reduced(const tg_grid* grid, const double* youngs_per_voxel, double poisson,
                     const tg_dirichlet_bc* bcs, int32_t nbc, const tg_nodal_load* loads,
                     int32_t nloads, uint8_t* kept, double* rhs, double* invdiag,
                     int32_t* ng_out);

/* fea_solve_mgcg_matfree (graded overload, core/include/topopt/fea.hpp:707-715;
 * core/src/fea/multigrid.cpp:2098-2320): solves the reduced, void-gated system
 * to ||b - A x|| <= tolerance ||b||, MG-PCG with a Jacobi-PCG fallback.
 * active_mask (one byte per voxel, 0 removes the element) and initial_guess
 * (ndof) may be NULL.  u_out receives the full ndof field. */
int tg_solve(const tg_grid* grid, const double* youngs_per_voxel, double poisson,
             const tg_dirichlet_bc* bcs, int32_t nbc, const tg_nodal_load* loads,
             int32_t nloads, double tolerance, int32_t max_iterations,
             const tg_solve_options* options, const uint8_t* active_mask,
             const double* initial_guess, double* u_out, tg_cg_info* info);

/* simp_compliance (core/include/topopt/simp.hpp:247-255; simp.cpp:567-828):
 * the penalised solve, c = sum E(rho_e) q_e and dc/drho.  u_out (ndof) and
 * dc_out (voxels) may be NULL. */
int tg_simp_compliance(const tg_grid* grid, const tg_simp_params* params,
                       const double* density, const tg_dirichlet_bc* bcs, int32_t nbc,
                       const tg_nodal_load* loads, int32_t nloads, double tolerance,
                       int32_t max_iterations, const tg_solve_options* options,
                       double* u_out, double* dc_out, double* compliance_out,
                       tg_cg_info* info);

/* DensityFilter::filter_density / filter_sensitivity over the solid voxels
 * (core/src/simp/simp.cpp:834-942); radius in voxel units.  adjoint 0 = forward. */
int tg_filter(const tg_grid* grid, double radius, int32_t adjoint, const double* x,
              double* out);

/* oc_update (core/include/topopt/simp.hpp:481-485; simp.cpp:948-1025): the OC
 * step with the lambda bisection on the filtered volume.  Bit-identical to the
 * reference for the same inputs. */
int tg_oc_update(const tg_grid* grid, double radius, const double* density,
                 const double* dcompliance, double volume_fraction, double move,
                 double density_min, double* x_new);

/* ---- active domain (the restricted-analysis mask) ----
 * active_domain_auto_band (simp.hpp:314; simp.cpp:440-447): ceil(filter_radius) + 1,
 * 1 for a non-finite or non-positive radius.  Host only. */
int32_t tg_active_domain_auto_band(double filter_radius);

/* active_domain_mask (simp.hpp:298-300; simp.cpp:449-528), on the device:
 * mask_out[e] = 1 iff voxel e is solid and within Chebyshev distance `band` of
 * a core voxel (solid with density > 1.5 density_min, or tagged Load 4 / Fixture
 * 5); band <= 0 returns every solid voxel.  Integer-exact: bit-identical to the
 * reference for the same inputs.  active_count (may be NULL) receives the number
 * of ones. */
int tg_active_domain_mask(const tg_grid* grid, const double* density, double density_min,
                          int32_t band, uint8_t* mask_out, int64_t* active_count);

/* active_domain_escape_count (simp.hpp:336-339; simp.cpp:530-556), on the
 * device: solid voxels outside prev_mask whose density exceeds 1.5 density_min;
 * 0 when prev_mask is NULL (the first armed iteration). */
int tg_active_domain_escape_count(const tg_grid* grid, const double* density,
                                  const uint8_t* prev_mask, double density_min,
                                  int64_t* escapes);

/* ---- design masks (passive regions) ----
 * Mask bytes are MaskValue (core/include/topopt/voxel.hpp:42-46): 0 Active,
 * 1 FrozenSolid, 2 FrozenVoid, one per voxel; other values are rejected. */

/* effective_design_mask (simp.hpp:462; simp.cpp:2610-2633): Empty voxels become
 * FrozenVoid, Load (tag 4) and Fixture (tag 5) voxels FrozenSolid. */
int tg_effective_design_mask(const tg_grid* grid, const uint8_t* mask, uint8_t* eff_out);

/* The mask-aware density filter, make_density_filter(grid, radius, mask)
 * (simp.hpp:444-446; simp.cpp:834-890) with one forward or adjoint pass: only
 * solid voxels whose mask entry is Active are filter voxels. */
int tg_filter_masked(const tg_grid* grid, const uint8_t* mask, double radius, int32_t adjoint,
                     const double* x, double* out);

/* oc_update_masked (simp.cpp:2662-2720) under the effective mask of `mask` and
 * its Active-only filter: only Active voxels move, frozen voxels keep their x,
 * the budget is volume_fraction * (Active voxels).  Bit-identical. */
int tg_oc_update_masked(const tg_grid* grid, const uint8_t* mask, double radius,
                        const double* density, const double* dcompliance,
                        double volume_fraction, double move, double density_min,
                        double* x_new);

/* heaviside_project and heaviside_project_derivative (simp.hpp:506-514;
 * simp.cpp:352-365) of n values of rho_tilde, on the device: value and
 * derivative may each be NULL.  beta must be finite and > 0, eta in (0, 1).
 * Computed with the device's tanh and cosh, so within a few units in the last
 * place of the host library's values. */
int tg_heaviside_project(int64_t n, const double* rho_tilde, double beta, double eta,
                         double* value, double* derivative);

/* heaviside_continuation_schedule (simp.hpp:530; simp.cpp:367-374): the locked
 * six-stage schedule, beta 1 -> 32 doubling, 50 iterations each, move 0.2 up to
 * beta 8, 0.1 at 16, 0.05 at 32.  Writes min(cap, 6) stages to out (may be NULL
 * with cap 0) and returns 6. */
int32_t tg_heaviside_continuation_schedule(tg_projection_stage* out, int32_t cap);

/* oc_update_projected (simp.cpp:1665-1726): the projection derivative at xtilde
 * (= filter(density)) chained before the filter transpose for dc and dv, the
 * ratio -dc/(lambda dv) with unclamped dv (a non-finite ratio holds the voxel),
 * and the bisection on the projected volume sum heaviside_project(filter(x_new))
 * over the solid voxels. */
int tg_oc_update_projected(const tg_grid* grid, double radius, const double* density,
                           const double* xtilde, const double* dcompliance, double beta,
                           double eta, double volume_fraction, double move, double density_min,
                           double* x_new);

/* simp_optimize (core/include/topopt/simp.hpp:1783-1786; simp.cpp:2018-2592):
 * the OC loop, unprojected or with a beta-continuation plan in
 * options->projection.  history (max_iterations rows, or the plan's total
 * iterations), design_out and phys_out (voxels) may be NULL; cancel (may be
 * NULL) is polled once per iteration, before the solve (simp.cpp:2161). */
int tg_simp_optimize(const tg_grid* grid, const tg_simp_params* params,
                     const tg_dirichlet_bc* bcs, int32_t nbc, const tg_nodal_load* loads,
                     int32_t nloads, const tg_simp_options* options, tg_progress_fn progress,
                     void* progress_ctx, const volatile int32_t* cancel,
                     tg_simp_iteration* history, double* design_out, double* phys_out,
                     tg_simp_result* result);

/* The masked overload, simp_optimize(grid, params, bcs, loads, options, mask)
 * (simp.hpp:1820-1824; simp.cpp:2989-3640), OC with or without projection (the
 * projection acts on the Active voxels, project_active simp.cpp:2789): the analysis
 * grid drops FrozenVoid voxels, the physical density is pinned (FrozenSolid 1,
 * FrozenVoid 0) before each solve and in phys_out, and volume fractions are
 * over the Active voxels. */
int tg_simp_optimize_masked(const tg_grid* grid, const tg_simp_params* params,
                            const tg_dirichlet_bc* bcs, int32_t nbc, const tg_nodal_load* loads,
                            int32_t nloads, const tg_simp_options* options, const uint8_t* mask,
                            tg_progress_fn progress, void* progress_ctx,
                            const volatile int32_t* cancel, tg_simp_iteration* history,
                            double* design_out, double* phys_out, tg_simp_result* result);

/* ---- stress, strength margins and the volume-fraction ladder ---- */

/* The strength side of analyze_fixed_design (analyze.cpp:145-440) in its
 * solid-material posture: Material::yield_strength_mpa and z_knockdown, the
 * build direction, the printed-set threshold, KnockdownSpec::infill_knockdown
 * and the acceptance threshold. */
typedef struct {
  double yield_strength;   /* finite, > 0 */
  double z_knockdown;      /* (0, 1] */
  double build_dir[3];     /* non-zero; normalised internally */
  double printed_iso;      /* printed voxels: density > printed_iso, in (0, 1) (0.5) */
  double infill_knockdown; /* scales the worst-case margin at the gate (1 = solid) */
  double margin_stop;      /* accepted: margin_effective >= margin_stop (finite, >= 0) */
} tg_strength_spec;

typedef struct {
  int32_t non_convergent;  /* the certification solve failed: never accepted */
  int32_t cg_iterations, load_path_ok, accepted;
  int64_t printed_voxels;
  double compliance, max_von_mises, max_interlayer_tension;
  double margin_in_plane, margin_interlayer, margin_worst_case, margin_effective;
} tg_fixed_design_analysis;

/* The stress field of a displacement (hex8_stress, hex_element.cpp:242-316, at
 * each voxel's centre, on the device): for every solid voxel whose density
 * exceeds iso (density NULL: every solid voxel), the Cauchy stress (Voigt
 * xx,yy,zz,xy,yz,zx, true shear) into sigma_out[6 e..] and von Mises into
 * von_mises_out[e]; other voxels 0.  u has 3 (nx+1)(ny+1)(nz+1) entries.  Either
 * output may be NULL.  Rounds exactly like the reference. */
int tg_element_stress(const tg_grid* grid, double youngs_modulus, double poisson,
                      const double* u, const double* density, double iso, double* sigma_out,
                      double* von_mises_out);

/* load_path_connected (voxel.hpp:359-361; voxelize.cpp:609-726): whether the
 * printed voxels (tag != Empty, density > iso) connect, 26-connected, every
 * Load (tag 4) voxel to a printed Fixture (tag 5) voxel; vacuously 1 without
 * Load or Fixture voxels. */
int tg_load_path_connected(const tg_grid* grid, const double* density, double iso,
                           int32_t* connected);

/* analyze_fixed_design, solid posture: the certification solve of the fixed
 * density at cg_tolerance (a failure sets non_convergent and returns TG_OK),
 * the stress of every printed voxel with the SOLID modulus, the peak von Mises
 * and interlayer tension max(0, n.sigma.n) along the build direction,
 * compute_stress_margin (report.cpp:464-491), the load-path belt and the gate.
 * von_mises_out (nv), stress_out (6 nv) and displacement_out (3 (nx+1)(ny+1)(nz+1):
 * the solve's displacement at the nodes of printed voxels, 0 elsewhere,
 * analyze.cpp:385-394) may be NULL. */
int tg_analyze_fixed_design(const tg_grid* grid, const tg_simp_params* params,
                            const double* density, const tg_dirichlet_bc* bcs, int32_t nbc,
                            const tg_nodal_load* loads, int32_t nloads,
                            const tg_strength_spec* strength, double cg_tolerance,
                            int32_t cg_max_iterations, const tg_solve_options* solve,
                            tg_fixed_design_analysis* out, double* von_mises_out,
                            double* stress_out, double* displacement_out);

/* self_weight_loads (fea.hpp:215; assembly.cpp) and its masked form
 * (minimize_plastic.cpp:132-143, FrozenVoid voxels weigh nothing): gravity *
 * density * voxel volume / 8 on each corner node of every solid voxel along the
 * unit direction, one load per (node, non-zero component) in node order.
 * Writes min(count, cap) loads to out (may be NULL with cap 0) and returns the
 * count, or -1 on invalid arguments (tg_last_error). */
int64_t tg_self_weight_loads(const tg_grid* grid, const uint8_t* mask, double density,
                             double gravity, const double direction[3], tg_nodal_load* out,
                             int64_t cap);

/* The volume-fraction ladder of minimize_plastic (pipeline.hpp:113-1060;
 * minimize_plastic.cpp:1402-2742) for the OC updater, without lattice, design
 * box or product options: volume_fractions strictly descending in (0, 1]. */
typedef struct {
  const double* volume_fractions;
  int32_t rungs;
  int32_t warm_start_inherit; /* seed each rung from the last connected rung's density */
  tg_strength_spec strength;
} tg_ladder_options;

typedef struct {
  double volume_fraction;
  int32_t trajectory_ok; /* 0: infeasible or non-convergent trajectory, not analysed */
  int32_t analysed;      /* the certification solve converged */
  int32_t accepted;
  tg_simp_result optimization;
  tg_fixed_design_analysis analysis;
} tg_ladder_rung;

typedef struct {
  int32_t evaluated;         /* rungs run */
  int32_t recommended;       /* the last accepted rung (the lightest that passed), or -1 */
  int32_t stopped_on_margin; /* a rung's margin fell below margin_stop */
  int32_t cancelled;
} tg_ladder_result;

/* The ladder walk: rung r runs the masked simp_optimize at volume_fractions[r]
 * (mask NULL: every voxel Active), seeded from the warm seed; an infeasible or
 * non-convergent trajectory is rejected unanalysed and the walk continues; a
 * connected rung becomes the seed (warm_start_inherit) ; the analysis on the
 * caller's grid; a rejected rung stops the walk only when its margin failed.
 * rungs_out has room for ladder->rungs entries; design_out / phys_out receive
 * the recommended rung's fields (untouched when none was accepted). */
int tg_minimize_plastic(const tg_grid* grid, const tg_simp_params* params,
                        const tg_dirichlet_bc* bcs, int32_t nbc, const tg_nodal_load* loads,
                        int32_t nloads, const tg_simp_options* simp, const uint8_t* mask,
                        const tg_ladder_options* ladder, tg_progress_fn progress,
                        void* progress_ctx, const volatile int32_t* cancel,
                        tg_ladder_rung* rungs_out, tg_ladder_result* result, double* design_out,
                        double* phys_out);

/* ---- on-disk formats: design.bin, fields.bin, iterations.csv ---- */

/* The solved grid a container indexes to (VoxelGrid's dims, origin, spacing). */
typedef struct {
  int32_t nx, ny, nz;
  double origin[3];
  double spacing;
} tg_grid_frame;

/* One design.bin v1 variant block (design_store.hpp:44-78, StoredDesign
 * :111-128); density has nx*ny*nz entries. */
typedef struct {
  double requested_volume_fraction, achieved_volume_fraction;
  double margin_worst_case, margin_effective, max_von_mises;
  int32_t accepted, iterations;
  double applied_build_dir[3];
  int32_t build_direction_auto_applied, export_baked;
  uint64_t fingerprint; /* filled by the reader; the writer computes its own */
  const double* density;
} tg_design_variant;

/* design_fingerprint (design_store.hpp:102; design_store.cpp): FNV-1a 64 over
 * the density's little-endian bytes. */
uint64_t tg_design_fingerprint(const double* density, int64_t count);

/* write_design_file (design_store.hpp:154-181): the v1 container, written to
 * "<path>.part" and renamed onto path.  Returns the blocks written, or -1
 * (tg_last_error). */
int32_t tg_write_design_file(const char* path, const tg_grid_frame* frame,
                             const tg_design_variant* variants, int32_t count);

/* read_design_file (design_store.hpp:183): checks the version, the header, each
 * block's density count and fingerprint.  Fills frame and *count; the first
 * min(count, cap) variants go to variants_out with their densities copied into
 * density_out (cap * nx*ny*nz doubles) and pointed at there.  Either output
 * may be NULL with cap 0 (a header probe).  Returns TG_OK or TG_EINVAL. */
int tg_read_design_file(const char* path, tg_grid_frame* frame, int32_t* count,
                        tg_design_variant* variants_out, int32_t cap, double* density_out);

/* One fields.bin v1 block (fields.hpp:40-75): the per-voxel von Mises (nx*ny*nz)
 * and per-node displacement (3 (nx+1)(ny+1)(nz+1)), narrowed to float32 on
 * write; the stress tensor is absent in v1. */
typedef struct {
  double requested_volume_fraction, mass_grams;
  int32_t support_volume_voxels;
  const double* von_mises;
  const double* displacement;
} tg_fields_variant;

/* write_fields_file (fields.hpp:96-118) over the blocks given (the caller picks
 * the accepted variants).  Returns the blocks written, or -1. */
int32_t tg_write_fields_file(const char* path, const tg_grid_frame* frame,
                             const tg_fields_variant* variants, int32_t count);

/* One iterations.csv row (observability.hpp:72-184; SimpIterationObservation,
 * simp.hpp:920-1000, with IterationPhaseTimes :873-918). */
typedef struct {
  int32_t iteration;
  double compliance, volume_fraction;
  int32_t plateau, cg_iterations, cg_multigrid;
  double beta;
  int32_t hier_built, mg_cycles_attempted, infeasible, recycle_dim;
  double active_fraction;
  double total_ms, tail_prev_ms, filter_ms, project_ms, solve_ms, fea_ms, sens_ms, update_ms,
      analysis_ms, observe_ms, residual_ms;
  double solver_build_ms, mg_build_ms, mg_ms, cg_ms, geneo_setup_ms, geneo_apply_ms, recycle_ms;
  int64_t fea_solves, matvecs;
  int32_t geneo_dim, geneo_action, geneo_burn, geneo_threshold;
  double rss_mb, peak_rss_mb, compressed_mb, available_mb;
  int64_t major_faults, swapins;
} tg_iteration_record;

/* kIterationCsvHeader (observability.cpp:252-264), without the newline. */
const char* tg_iteration_csv_header(void);
/* The record of one library iteration: the solve and update phases from the
 * row's timings, the rest at the reference's "absent" values (memory -1). */
void tg_iteration_record_from(const tg_simp_iteration* row, int32_t infeasible,
                              tg_iteration_record* out);
/* IterationCsvWriter::append_at's row (observability.cpp:282-331), newline
 * included, into buf; returns its length (or the length needed when cap is too
 * small, buf then untouched). */
int64_t tg_iteration_csv_row(int64_t rung, const tg_iteration_record* rec, int64_t wall_ms,
                             char* buf, int64_t cap);

/* ---- periodic homogenization of unit cells ---- */
typedef struct {
  int32_t iterations_max;    /* largest CG iteration count over the batch */
  int32_t converged;         /* 1 when every system met the tolerance */
  int32_t systems;           /* cells x solved strain columns */
  int64_t iterations_total;  /* sum of the CG iteration counts (inner ones, mixed) */
  int32_t refinements;       /* mixed: FP64 refinement steps */
  double t_setup_ms, t_solve_ms, t_total_ms;
} tg_homog_info;

/* Periodic strain homogenization of a batch of unit cells, the homogenize()
 * of core/tests/harness/lattice_homog_probe.cpp:290-412 (a harness library;
 * no production caller): cells of nx*ny*nz voxels with opposite faces
 * identified, tags ncell*nx*ny*nz bytes (cell c at c*nx*ny*nz, 0 = void,
 * voids carry no element), Hex8 elements of modulus E, Poisson nu, edge
 * spacing.  cases_mask selects the Voigt strain columns [xx,yy,zz,gxy,gyz,gzx]
 * solved (bit J; 0x3F = all six).  Each system is solved by Jacobi-PCG to
 * |r| < tolerance |b| (max_iterations <= 0: min(2 ndof, 200000)); precision
 * TG_PREC_MIXED runs FP32 inner Jacobi-PCG solves (relative 1e-3) inside FP64
 * iterative refinement judged on the FP64 residual.  ch_out
 * receives ncell 6x6 tensors, row-major, CH[I][J] filled for the solved
 * columns J (others 0).  TG_ENONCONV when a system missed the tolerance (the
 * tensors are still written). */
int tg_homogenize(int32_t ncell, int32_t nx, int32_t ny, int32_t nz, double spacing,
                  double youngs_modulus, double poisson, const uint8_t* tags,
                  int32_t cases_mask, double tolerance, int32_t max_iterations,
                  int32_t precision, double* ch_out, tg_homog_info* info);

/* How host threads wait for the GPU (this process, the current device): 0 the
 * CUDA default, 1 spin, 2 yield, 3 block on a synchronisation primitive.  Many
 * concurrent jobs on few host cores wait better with 2 or 3. */
int tg_set_sync_mode(int32_t mode);

/* ---- serving: continuous batching of optimisation jobs ----
 * No reference counterpart as one interface: the GB300 form of the callers that
 * run simp_optimize once per request (minimize_plastic, the app bridge,
 * TopOptBridge.hpp:262-269).  Jobs queue in arrival order and are admitted,
 * head first, when a slot is free and their device-memory estimate
 * (tg_job_estimate_bytes) fits in the remaining HBM budget; each admitted job
 * runs tg_simp_optimize(_masked) on its own worker thread and CUDA stream, so
 * the jobs in flight overlap on the GPU, and a job's result is the same alone
 * and in the mix. */
typedef struct tg_server tg_server;
typedef struct {
  int64_t hbm_budget_bytes; /* admission budget: sum of the admitted jobs' estimates */
  int32_t max_active;       /* concurrent jobs (worker threads), >= 1 */
  int32_t device;           /* CUDA device ordinal */
} tg_server_config;
typedef struct {
  int64_t ticket;
  int32_t status;           /* the job's tg_simp_optimize status */
  int64_t estimate_bytes;
  double t_queue_ms;        /* submission to admission */
  double t_run_ms;          /* admission to completion */
  double t_latency_ms;      /* submission to completion */
  tg_simp_result result;
} tg_server_result;
typedef struct {
  int64_t submitted, admitted, completed, rejected, queued;
  int32_t active, peak_active;
  int64_t bytes_in_use, peak_bytes;
  double uptime_ms, busy_ms; /* busy: time with at least one job running */
} tg_server_counters;

int tg_server_create(const tg_server_config* cfg, tg_server** out);
/* Copies the problem; TG_ENOMEM when its estimate exceeds the whole budget. */
int tg_server_submit(tg_server* server, const tg_grid* grid, const tg_simp_params* params,
                     const tg_dirichlet_bc* bcs, int32_t nbc, const tg_nodal_load* loads,
                     int32_t nloads, const tg_simp_options* options, const uint8_t* mask,
                     int64_t* ticket_out);
/* Blocks until the job is done; returns its status and releases the ticket
 * (a later wait on it returns TG_EINVAL).  design_out / phys_out (voxels) may
 * be NULL. */
int tg_server_wait(tg_server* server, int64_t ticket, tg_server_result* out,
                   double* design_out, double* phys_out);
int tg_server_stats(tg_server* server, tg_server_counters* out);
/* Drops queued jobs (their waiters return TG_EINVAL), waits for the admitted
 * ones, frees the server.  No other call on the server may be in flight or
 * follow. */
void tg_server_destroy(tg_server* server);

/* ---- resident jobs: state stays on the device between design iterations ---- */
typedef struct tg_job tg_job;

/* Set up a job (grid, filter, BC mask, hierarchy structure) and its uniform start
 * design; no design iteration runs. */
int tg_job_create(const tg_grid* grid, const tg_simp_params* params,
                  const tg_dirichlet_bc* bcs, int32_t nbc, const tg_nodal_load* loads,
                  int32_t nloads, const tg_simp_options* options, tg_job** job_out);
/* tg_job_create for the masked overload (see tg_simp_optimize_masked). */
int tg_job_create_masked(const tg_grid* grid, const tg_simp_params* params,
                         const tg_dirichlet_bc* bcs, int32_t nbc, const tg_nodal_load* loads,
                         int32_t nloads, const tg_simp_options* options, const uint8_t* mask,
                         tg_job** job_out);
/* One design iteration on the device: filter, solve, sensitivities, OC update
 * (projected, at the current stage's beta and move, when the options carry a
 * projection plan). */
int tg_job_step(tg_job* job, tg_simp_iteration* row);
/* Select the stage of the options' projection plan the next steps run
 * (0 <= stage < projection_stages; stage 0 at creation). */
int tg_job_set_stage(tg_job* job, int32_t stage);
/* Copy the current design x and physical density (filter(x), projected at the
 * current stage's beta, pinned for masked jobs) to the host. */
int tg_job_read(tg_job* job, double* design_out, double* phys_out);
/* Copy the displacement of the job's last solve (ndof, the full field with the
 * prescribed values on fixed DOFs; zeros before the first step) to the host:
 * the warm start the next step's solve begins from (simp.cpp:1788-1797). */
int tg_job_read_displacement(tg_job* job, double* u_out);
/* Replace the design with a host field (voxels). */
int tg_job_write_design(tg_job* job, const double* design);
/* Page-locked host memory for the host buffers of the calls above: their copies
 * from and to such a buffer run as direct DMA instead of through a staging
 * copy.  NULL when the allocation fails; free with tg_host_free (NULL is a
 * no-op). */
void* tg_host_alloc(int64_t bytes);
int tg_host_free(void* ptr);
/* Bytes of device memory the job holds. */
int64_t tg_job_device_bytes(const tg_job* job);
/* Estimate, before creating it, the device bytes a job on this grid needs. */
int64_t tg_job_estimate_bytes(const tg_grid* grid, const tg_simp_options* options);
void tg_job_destroy(tg_job* job);

/* ---- the density filter without device allocation ----
 * No counterpart in the reference: an addition for callers that cannot call
 * cudaMalloc when they filter (allocator-free serving or real-time loops, hosts
 * whose device memory belongs to another runtime's arena).  Same result as
 * tg_filter, bit for bit; inputs and outputs are the caller's DEVICE buffers
 * (d_tags: one VoxelTag byte per voxel, NULL = all solid; d_x, d_out: voxels),
 * enqueued on `stream` (a cudaStream_t, NULL = the legacy default stream) and
 * not synchronised.  Scratch lives in one fixed device array of the library:
 * at most 1,048,576 voxels and a radius of at most 6 voxels (TG_EINVAL beyond);
 * every GPU that loads the library holds the array (~17 MB) until exit.  Calls
 * share it, so calls that overlap on the GPU race -- keep them on one stream.
 * Every call looks up the array's address in the current device's context, so
 * it stays valid across cudaDeviceReset; the first call on a device may load
 * the library's module there (make it before any stream capture).  No call
 * allocates, frees or leaves state for the next. */
int tg_filter_noalloc(int32_t nx, int32_t ny, int32_t nz, const uint8_t* d_tags, double radius,
                      int32_t adjoint, const double* d_x, double* d_out, void* stream);

/* ---- measurement (no reference counterpart) ---- */
/* Average device time of one fine-operator launch (y = A x on the job's current
 * element factors), precision TG_PREC_FP64, TG_PREC_MIXED (FP32) or TG_APPLY_DF
 * (the double-float residual kernel), or of one level-1 operator launch of a
 * mixed job (TG_APPLY_L1_STENCIL, TG_APPLY_L1_TC), over `reps` back-to-back
 * launches timed with CUDA events on the job's stream. */
int tg_job_time_operator(tg_job* job, int32_t precision, int32_t reps, double* avg_ms);
/* The level-1 operator of a mixed job's V-cycle on its current design, applied
 * to a seeded vector by the assembled FP32 stencil and by the tensor-core
 * operator: max |difference| / max |stencil result|. */
int tg_job_check_level1(tg_job* job, double* rel_diff);
/* Kernels this library has launched in the process so far. */
int64_t tg_kernel_launches(void);
/* Level 1 of the mixed form's V-cycle: on (default) the Galerkin operator is
 * applied on the tensor cores from the fine moduli (tcgen05, TF32 splits to
 * FP32 accuracy); off, as the assembled FP32 node stencil.  Applies to solvers
 * created afterwards. */
int tg_set_level1_tc(int32_t on);
/* Level 1's Galerkin matrices in the mixed form with level 1 on the tensor
 * cores: on (default) the fast-path elements' matrices (sum_c E_c G_c) come
 * from a bandwidth-bound kernel, the others from the general one; off, all from
 * the general one.  The matrices are bit-identical either way.  Applies to
 * hierarchy builds from then on. */
int tg_set_level1_galerkin_fast(int32_t on);
/* The mixed form's V-cycle on its small levels (below level 1, from the first
 * level of at most 4096 nodes to the coarsest): on, they run as one launch of
 * one thread-block cluster with the cluster barrier between steps; off
 * (default), as a launch per step, which measured faster on GB300.  Same
 * arithmetic either way.  Applies to solvers created afterwards. */
int tg_set_coarse_fused(int32_t on);
/* Schedule of the FP32 fine operator (the mixed form's fine level).  kind 0:
 * the pencil kernel; kind 1: the column-blocked kernel with tile shape `shape`
 * (0 <= shape < 8: Y x W element rows per thread x warps per CTA of 4x4, 6x4,
 * 3x4, 2x8 for shapes 0-3, the same tiles with the x and y components in
 * paired FP32 instructions for shapes 4-7) and `kz` >= 8 element layers per
 * CTA.  The setting overrides the per-grid, per-mode table (apply, residual,
 * smoothing; measured on the first large mixed job of a grid) for every later
 * FP32 launch in the process; kind < 0 clears it.  Results of every schedule
 * agree to FP32 rounding. */
int tg_set_fp32_schedule(int32_t kind, int32_t shape, int32_t kz);
/* The FP32 schedule the operator's apply mode uses on an nx x ny x nz grid now. */
int tg_fp32_schedule(int32_t nx, int32_t ny, int32_t nz, int32_t* kind, int32_t* shape,
                     int32_t* kz);
/* FMA microbenchmark: sustained FP64 and FP32 FMA throughput of the device in
 * TFLOP/s (2 flops per FMA), all SMs, register-resident operands. */
int tg_device_fma_peaks(double* fp64_tflops, double* fp32_tflops);

#ifdef __cplusplus
}
#endif
#endif
