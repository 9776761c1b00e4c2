/*
 * topopt_oracle.h -- CPU restatement of the reference voxel-SIMP inner loop.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: it is linked by the
 * tests, by __graft_entry__.smoke() and by bench.py's CPU-baseline leg, never by
 * the product library (topopt_gb300/csrc).  Every function restates one piece of
 * the reference algorithm (Anarkissed/TopOpt, core/) in plain C, in the same
 * arithmetic order where the reference fixes one, and cites the file:line it
 * follows.  Compile with -ffp-contract=off so no multiply/add pair is fused; the
 * reference uses explicit mul+add for the same reason (core/src/fea/matfree.cpp:66-73).
 *
 * Parity pin: the restatement is checked against (1) the reference's own Ke
 * fixture core/tests/fixtures/fea/hex_stiffness_reference.json and (2) golden
 * vectors produced by the reference's own compiled code (oracle/_ref, built by
 * oracle/build_ref.sh) and committed under tests/golden/.
 *
 * Conventions (core/include/topopt/fea.hpp:18-29, :153-171):
 *   voxel (i,j,k)  -> e = (k*ny + j)*nx + i               (x fastest)
 *   node  (a,b,c)  -> n = (c*(ny+1) + b)*(nx+1) + a
 *   DOF            -> 3*n + comp                          (node-major interleaved)
 *   Hex8 local node order: bottom face CCW then top face CCW.
 * `solid` is one byte per voxel (non-zero = solid, i.e. VoxelTag != Empty); NULL
 * means every voxel is solid.
 */
#ifndef TOPOPT_ORACLE_H
#define TOPOPT_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { OR_OK = 0, OR_EINVAL = 1, OR_ESINGULAR = 2, OR_ENONCONV = 3 };

/* Host threads the oracle's parallel loops use (1 when built without OpenMP). */
int or_threads(void);
/* Sets the thread count of later parallel loops (n > 0; a no-op without
 * OpenMP).  Launchers such as torchrun export OMP_NUM_THREADS=1; a timed CPU
 * run sets the count it means to use. */
void or_set_threads(int n);

/* Last error message of the calling thread ("" when none). */
const char* or_last_error(void);

/* 24x24 row-major element stiffness, 2x2x2 Gauss (hex_element.cpp:23-115). */
int or_hex8_stiffness(double E, double nu, double h, double* ke576);

/* y = K u over the full grid; factor == NULL -> uniform modulus E baked into Ke,
 * else Ke(E=1) and factor[e] per solid voxel (matfree.cpp:1079-1098, :535-553).
 * Colour-ordered element loop with the reference's column-major mul+add. */
int or_apply(int nx, int ny, int nz, double h, const uint8_t* solid,
             const double* factor, double E, double nu, const double* u, double* y);

/* The same apply with a caller-computed unit-modulus Ke (or_hex8_stiffness) and
 * factors already checked (> 0 on solid voxels). */
void or_apply_ke(int nx, int ny, int nz, const uint8_t* solid, const double* factor,
                 const double* ke576, const double* u, double* y);

/* Reduced, void-gated system (matfree.cpp:670-834).  Outputs (all ndof long):
 *   kept[d]   1 if DOF d survives (free and touched by a solid element)
 *   rhs[d]    f - K u_p on kept DOFs, 0 elsewhere
 *   invdiag[d] 1/diag on kept DOFs, 0 elsewhere
 *   up[d]     prescribed displacement field
 * Returns OR_ESINGULAR for a void-only system or a load on a void DOF. */
int or_build_reduced(int nx, int ny, int nz, double h, const uint8_t* solid,
                     const double* factor, double E, double nu,
                     int nbc, const int* bc_node, const int* bc_comp, const double* bc_val,
                     int nload, const int* ld_node, const int* ld_comp, const double* ld_val,
                     uint8_t* kept, double* rhs, double* invdiag, double* up, int* ng_out);

/* Jacobi-PCG solve of the reduced system, Eigen-criterion (matfree.cpp:841-1076,
 * 1106-1170).  u (ndof) receives the full field.  initial_guess may be NULL. */
int or_solve_cg(int nx, int ny, int nz, double h, const uint8_t* solid,
                const double* factor, double E, double nu,
                int nbc, const int* bc_node, const int* bc_comp, const double* bc_val,
                int nload, const int* ld_node, const int* ld_comp, const double* ld_val,
                double tol, int max_it, const double* initial_guess,
                double* u, int* iters, double* resid);

/* SIMP compliance + sensitivities (simp.cpp:567-828): reference law
 * E = clamp(rho, rho_min, 1)^p * E0.  dc is 0 on non-solid voxels. */
int or_simp_compliance(int nx, int ny, int nz, double h, const uint8_t* solid,
                       double E0, double nu, double penal, double rho_min,
                       const double* density,
                       int nbc, const int* bc_node, const int* bc_comp, const double* bc_val,
                       int nload, const int* ld_node, const int* ld_comp, const double* ld_val,
                       double tol, int max_it, double* u, double* dc,
                       double* compliance, int* iters, double* resid);

/* Compliance + sensitivities from a given displacement field (the sweep of
 * simp.cpp:747-824 without the solve). */
int or_sensitivity(int nx, int ny, int nz, double h, const uint8_t* solid,
                   double E0, double nu, double penal, double rho_min,
                   const double* density, const double* u, double* dc,
                   double* compliance);

/* Density filter (simp.cpp:834-942): CSR over active design voxels.  `active`
 * (one byte per voxel, NULL = solid) selects the design voxels. */
typedef struct or_filter or_filter;
or_filter* or_filter_make(int nx, int ny, int nz, const uint8_t* solid,
                          const uint8_t* active, double radius);
void or_filter_free(or_filter* f);
size_t or_filter_nnz(const or_filter* f);
void or_filter_weight_sum(const or_filter* f, double* hs);
void or_filter_density(const or_filter* f, const double* x, double* out);
void or_filter_sensitivity(const or_filter* f, const double* s, double* out);

/* OC update with lambda bisection (simp.cpp:948-1025).  Writes x_new; the final
 * lambda and the number of volume evaluations are returned for diagnostics. */
int or_oc_update(int nx, int ny, int nz, const uint8_t* solid, const or_filter* f,
                 const double* density, const double* dc, double volfrac,
                 double move, double rho_min, double* x_new,
                 double* lambda_out, int* nvol_out);

/* MaskValue (core/include/topopt/voxel.hpp:42-46). */
enum { OR_ACTIVE = 0, OR_FROZEN_SOLID = 1, OR_FROZEN_VOID = 2 };

/* effective_design_mask (simp.cpp:2610-2633).  tags NULL = all Interior. */
void or_effective_design_mask(int nx, int ny, int nz, const uint8_t* tags, const uint8_t* mask,
                              uint8_t* eff);

/* oc_update_masked (simp.cpp:2662-2720): eff is an effective mask and f the
 * Active-only filter (or_filter_make with active = eff == Active). */
int or_oc_update_masked(int nx, int ny, int nz, const uint8_t* eff, const or_filter* f,
                        const double* density, const double* dc, double volfrac, double move,
                        double rho_min, double* x_new, double* lambda_out, int* nvol_out);

/* Plain simp_optimize with the OC updater (simp.cpp:2018-2592), with or
 * without a projection schedule.
 * The solve is the exact Jacobi-PCG above.  hist_* have room for max_it rows.
 * Guards: change_tol stop; rung-infeasibility window (simp.cpp:1140-1186) with
 * the reference defaults; non-convergence ends the run. */
typedef struct {
  double volume_fraction, filter_radius, move, change_tol, cg_tolerance;
  int max_iterations, cg_max_iterations;
  /* Heaviside projection schedule (SimpOptions::projection, simp.hpp:519-525,
   * :1443-1444): nstages = 0 is the unprojected loop; otherwise stage k runs
   * stage_iterations[k] OC iterations at (stage_beta[k], stage_move[k]). */
  int nstages;
  const double* stage_beta;
  const double* stage_move;
  const int* stage_iterations;
  double eta;
  /* Warm start (SimpOptions::initial_design, simp.hpp:1557-1575): NULL is the
   * uniform start; otherwise a raw seed density per voxel, rescaled to the
   * target mean over the design set, clamped and filtered once
   * (warm_start_design, simp.cpp:324-344). */
  const double* initial_design;
  /* The design updater (SimpOptions::updater, simp.hpp:1119): 0 OC, 1 MMA.
   * MMA stops a run on the objective plateau (mma_objective_plateau,
   * simp.cpp:1081-1134) when mma_plateau_window > 0, else on change_tol. */
  int updater;
  int mma_plateau_window;
  double mma_plateau_tol, mma_plateau_min_drop;
  int mma_plateau_flat_windows;
  /* Active domain (SimpOptions::active_domain_band, simp.hpp:1185-1227): 0 off,
   * > 0 the band, < 0 the auto band.  hist_active_fraction (output, may be NULL)
   * receives each iteration's active fraction (1 on the full domain). */
  int active_domain_band;
  double* hist_active_fraction;
} or_simp_options;

/* The MMA state across one run (MmaJointState): asymptotes and the last two
 * designs, nv each; iter the 1-based MMA iteration. */
typedef struct {
  double *low, *upp, *xold1, *xold2;
} or_mma_state;
/* mma_update / mma_update_masked (simp.cpp:1433-1489, :2736-2784) with the
 * subproblem mma_update_joint (mma_joint.cpp): design is the design set (solid
 * voxels, or Active voxels with the Active-only filter f). */
int or_mma_update(int nx, int ny, int nz, const uint8_t* design, const or_filter* f,
                  or_mma_state* st, int iter, const double* density, const double* dc,
                  double volfrac, double move, double rho_min, double* x_new,
                  double* lambda_out);
/* mma_objective_plateau (simp.cpp:1081-1134). */
int or_mma_objective_plateau(const double* c, int n, int window, double rel_tol, double min_drop,
                             int min_flat_windows);

/* The active domain: active_domain_auto_band (simp.cpp:440-447),
 * active_domain_mask (simp.cpp:449-528; tags NULL = every voxel Interior, Load 4
 * and Fixture 5 are pinned active), active_domain_escape_count
 * (simp.cpp:530-556; prev_mask NULL = 0). */
int or_active_domain_auto_band(double filter_radius);
int or_active_domain_mask(int nx, int ny, int nz, const uint8_t* tags, const double* density,
                          double density_min, int band, uint8_t* out);
long long or_active_domain_escape_count(int nx, int ny, int nz, const uint8_t* tags,
                                        const double* density, const uint8_t* prev_mask,
                                        double density_min);

/* heaviside_project and its derivative (simp.cpp:352-365). */
double or_heaviside_project(double rt, double beta, double eta);
double or_heaviside_project_derivative(double rt, double beta, double eta);
/* oc_update_projected (simp.cpp:1665-1726); xtilde = filter_density(density). */
int or_oc_update_projected(int nx, int ny, int nz, const uint8_t* solid, const or_filter* f,
                           const double* density, const double* xtilde, const double* dc,
                           double beta, double eta, double volfrac, double move,
                           double rho_min, double* x_new);
typedef struct {
  int iterations, converged, non_convergent, infeasible;
  double compliance, volume_fraction, initial_compliance;
  /* finalize_active_domain (simp.cpp:1981-1988). */
  int ad_band, ad_latched, ad_latch_iteration;
  long long ad_escape_count;
  double ad_fraction_mean;
  char ad_latch_reason[256];
} or_simp_result;
int or_simp_optimize(int nx, int ny, int nz, double h, const uint8_t* solid,
                     double E0, double nu, double penal, double rho_min,
                     int nbc, const int* bc_node, const int* bc_comp, const double* bc_val,
                     int nload, const int* ld_node, const int* ld_comp, const double* ld_val,
                     const or_simp_options* opt, double* hist_c, double* hist_change,
                     double* hist_vf, int* hist_cg, double* design, double* phys,
                     or_simp_result* res);

/* The masked simp_optimize overload (simp.cpp:2989-3640), OC, no projection:
 * tags are the voxel tags (0 Empty, 4 Load, 5 Fixture ...), mask the caller's
 * MaskValue per voxel.  phys receives the pinned physical density. */
int or_simp_optimize_masked(int nx, int ny, int nz, double h, const uint8_t* tags,
                            const uint8_t* mask, double E0, double nu, double penal,
                            double rho_min, int nbc, const int* bc_node, const int* bc_comp,
                            const double* bc_val, int nload, const int* ld_node,
                            const int* ld_comp, const double* ld_val, const or_simp_options* o,
                            double* hist_c, double* hist_change, double* hist_vf, int* hist_cg,
                            double* design, double* phys, or_simp_result* res);

/* ------------------------------------------------ stress and the ladder */
/* hex8_stress (hex_element.cpp:242-316): Cauchy stress (Voigt xx,yy,zz,xy,yz,zx,
 * true shear) and von Mises at natural coordinates (xi, eta, zeta) of a cubic
 * element with nodal displacements ue (24, hex8 order). */
int or_hex8_stress(double E, double nu, double h, const double* ue, double xi, double eta,
                   double zeta, double* sigma6, double* von_mises);
/* compute_stress_margin (settings/report.cpp:464-491): out = {in_plane,
 * interlayer, worst_case}; a zero stress is an unbounded (+inf) margin. */
int or_stress_margin(double yield_strength, double z_knockdown, double max_von_mises,
                     double max_interlayer, double* out3);
/* load_path_connected (voxelize.cpp:609-726): 26-connected flood fill over the
 * printed voxels (tag != Empty and density > iso) from the printed Fixture
 * (tag 5) voxels; 1 when it reaches every Load (tag 4) voxel, and vacuously 1
 * when the grid has no Load or no Fixture voxel.  tags NULL: no tags (1). */
int or_load_path_connected(int nx, int ny, int nz, const uint8_t* tags, const double* density,
                           double iso);

/* analyze_fixed_design (analyze.cpp:145-440), the solid-material posture: the
 * certification solve of the fixed density at cg_tol, the stress of every
 * printed voxel (solid, density > iso) at its centre with the SOLID modulus E0,
 * the peak von Mises and interlayer tension max(0, n.sigma.n) along build_dir,
 * the margins, the load-path belt, and accepted = load_path_ok && worst_case *
 * infill_knockdown >= margin_stop. */
typedef struct {
  int non_convergent, cg_iterations, load_path_ok, accepted;
  long long printed_voxels;
  double compliance, max_von_mises, max_interlayer;
  double margin_in_plane, margin_interlayer, margin_worst, margin_effective;
} or_analysis;
typedef struct {
  double yield_strength, z_knockdown, build_dir[3], iso, infill_knockdown, margin_stop;
} or_strength;
int or_analyze_fixed_design(int nx, int ny, int nz, double h, const uint8_t* tags, double E0,
                            double nu, double penal, double rho_min, const double* density,
                            int nbc, const int* bc_node, const int* bc_comp,
                            const double* bc_val, int nload, const int* ld_node,
                            const int* ld_comp, const double* ld_val, const or_strength* st,
                            double cg_tol, int cg_max_it, or_analysis* out, double* von_mises);

/* The ladder walk of minimize_plastic (minimize_plastic.cpp:1402-2742) for the
 * OC updater with no lattice, box or product options: rung r runs the masked
 * simp_optimize at volume_fraction ladder[r] (seeded from the warm seed), then
 *   cancelled/infeasible/non-convergent trajectory -> rejected, no analysis, the
 *     seed untouched, the walk continues;
 *   load_path_ok -> the seed becomes this rung's physical density when
 *     warm_start_inherit, else is cleared;
 *   the analysis; non-convergent certification -> rejected, continue;
 *   accepted -> recommended = r; else stop when the margin failed
 *     (stopped_on_margin), continue when only the load path did.
 * rungs_out[r] per evaluated rung; design/phys of the recommended rung. */
typedef struct {
  double volume_fraction;
  int iterations, trajectory_ok, analysed, accepted;
  double compliance;
  or_analysis analysis;
} or_rung;
int or_ladder(int nx, int ny, int nz, double h, const uint8_t* tags, const uint8_t* mask,
              double E0, double nu, double penal, double rho_min, int nbc, const int* bc_node,
              const int* bc_comp, const double* bc_val, int nload, const int* ld_node,
              const int* ld_comp, const double* ld_val, const or_simp_options* o,
              const double* ladder, int nrungs, int warm_start_inherit, const or_strength* st,
              or_rung* rungs_out, int* evaluated, int* recommended, int* stopped_on_margin,
              double* design, double* phys);

/* Periodic homogenization of one unit cell (lattice_homog_probe.cpp:290-412):
 * solid (NULL = all solid) selects the elements, cases_mask the Voigt strain
 * columns solved (bit J = column J; 0x3F all six), CH receives the 6x6 tensor
 * row-major (CH[I*6+J]; unsolved columns 0).  Jacobi-PCG at cg_tol, max_it <= 0
 * = min(2n, 200000). */
int or_homogenize(int nx, int ny, int nz, double h, double E, double nu, const uint8_t* solid,
                  int cases_mask, double cg_tol, int max_it, double* CH, int* iters_max,
                  int* converged);

/* ---- oracle_mg.c: the geometric-multigrid PCG, a labelled restatement ----
 * (multigrid.cpp:1211-1313 mf_mgpcg, :1344-1515 build_mf_hierarchy,
 * :557-697 build_hierarchy, :780-817 v_cycle, :1119-1146 mf_v_cycle): Galerkin
 * coarse operators as 27-point node stencils, damped Jacobi 0.6 with 1+1
 * sweeps, a banded Cholesky at the coarsest level (the reference: Eigen
 * SimplicialLDLT), coarsening until <= 6000 active DOFs (max_levels <= 0) or
 * exactly max_levels levels.  u = x on kept DOFs, u_p elsewhere. */
int or_mg_solve(int nx, int ny, int nz, double h, const uint8_t* solid, const double* factor,
                double nu, int nbc, const int* bc_node, const int* bc_comp, const double* bc_val,
                int nload, const int* ld_node, const int* ld_comp, const double* ld_val,
                double tol, int max_it, int max_levels, const double* initial_guess, double* u,
                int* iters, double* resid, int* levels);
/* niter design iterations of simp_optimize's OC loop with that solver, from the
 * design x (advanced in place); u: the displacement (a warm start on entry when
 * warm != 0).  Per iteration: compliance, MG-PCG iterations and seconds in
 * [filter + modulus, reduced system + hierarchy, MG-PCG, sensitivities, OC]. */
int or_design_iterations_mg(int nx, int ny, int nz, double h, const uint8_t* solid, double E0,
                            double nu, double penal, double rho_min, int nbc, const int* bc_node,
                            const int* bc_comp, const double* bc_val, int nload,
                            const int* ld_node, const int* ld_comp, const double* ld_val,
                            double volfrac, double radius, double move, double cg_tol,
                            int cg_max_it, int niter, int warm, double* x, double* u,
                            double* hist_c, int* hist_cg, double* hist_t5);

#ifdef __cplusplus
}
#endif
#endif
