// ref_capi.cpp -- flat extern "C" face over the reference's OWN compiled hot-path
// code (core/src/fea/hex_element.cpp, matfree.cpp, core/src/simp/simp.cpp), so the
// tests and the CPU baseline can call it through ctypes with the same argument
// layout as oracle/topopt_oracle.h.
//
// TEST INFRASTRUCTURE ONLY: the reference build is a checker and the timed CPU
// baseline; the product never links it.  Every entry point returns 0 on success,
// 1 for std::invalid_argument, 2 for std::runtime_error (void-gate rejections),
// 3 for SolverNonConvergence, 4 for anything else; ref_last_error() holds the
// exception text.
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include <array>

#include "fea/fea_matfree.hpp"
#include "topopt/design_store.hpp"
#include "topopt/fea.hpp"
#include "topopt/fields.hpp"
#include "topopt/observability.hpp"
#include "topopt/pipeline.hpp"
#include "topopt/orient.hpp"
#include "topopt/report.hpp"
#include "topopt/simp.hpp"
#include "topopt/voxel.hpp"

using namespace topopt;

namespace {
thread_local std::string g_err;

VoxelGrid make_grid(int nx, int ny, int nz, double h, const uint8_t* solid) {
  VoxelGrid g;
  g.nx = nx;
  g.ny = ny;
  g.nz = nz;
  g.spacing = h;
  const std::size_t nv = static_cast<std::size_t>(nx) * ny * nz;
  g.tags.assign(nv, VoxelTag::Interior);
  if (solid)
    for (std::size_t e = 0; e < nv; ++e)
      if (!solid[e]) g.tags[e] = VoxelTag::Empty;
  return g;
}

// A grid with the caller's raw tags (VoxelTag values; NULL = all Interior).
VoxelGrid make_grid_tags(int nx, int ny, int nz, double h, const uint8_t* tags) {
  VoxelGrid g = make_grid(nx, ny, nz, h, nullptr);
  if (tags)
    for (std::size_t e = 0; e < g.tags.size(); ++e) g.tags[e] = static_cast<VoxelTag>(tags[e]);
  return g;
}

DesignMask make_mask(std::size_t nv, const uint8_t* mask) {
  DesignMask m(nv);
  for (std::size_t e = 0; e < nv; ++e) m[e] = static_cast<MaskValue>(mask[e]);
  return m;
}

std::vector<DirichletBC> make_bcs(int n, const int* node, const int* comp, const double* val) {
  std::vector<DirichletBC> v(static_cast<std::size_t>(n));
  for (int i = 0; i < n; ++i) v[i] = DirichletBC{node[i], comp[i], val[i]};
  return v;
}

std::vector<NodalLoad> make_loads(int n, const int* node, const int* comp, const double* val) {
  std::vector<NodalLoad> v(static_cast<std::size_t>(n));
  for (int i = 0; i < n; ++i) v[i] = NodalLoad{node[i], comp[i], val[i]};
  return v;
}

template <class F>
int guarded(F&& fn) {
  try {
    fn();
    g_err.clear();
    return 0;
  } catch (const SolverNonConvergence& e) {
    g_err = e.what();
    return 3;
  } catch (const std::invalid_argument& e) {
    g_err = e.what();
    return 1;
  } catch (const std::runtime_error& e) {
    g_err = e.what();
    return 2;
  } catch (const std::exception& e) {
    g_err = e.what();
    return 4;
  }
}
}  // namespace

extern "C" {

const char* ref_last_error(void) { return g_err.c_str(); }

int ref_set_threads(int n) { return fea_set_matfree_threads(n); }

int ref_hex8_stiffness(double E, double nu, double h, double* ke) {
  return guarded([&] {
    const Hex8Stiffness K = hex8_stiffness(E, nu, h);
    std::memcpy(ke, K.k.data(), sizeof(double) * 576);
  });
}

int ref_apply(int nx, int ny, int nz, double h, const uint8_t* solid, const double* factor,
              double E, double nu, const double* u, double* y) {
  return guarded([&] {
    const VoxelGrid g = make_grid(nx, ny, nz, h, solid);
    const std::size_t ndof = 3 * static_cast<std::size_t>(fea_node_count(g));
    std::vector<double> uv(u, u + ndof), yv;
    if (factor) {
      std::vector<double> fv(factor, factor + g.voxel_count());
      yv = fea_matfree_apply(g, fv, nu, uv);
    } else {
      yv = fea_matfree_apply(g, E, nu, uv);
    }
    std::memcpy(y, yv.data(), ndof * sizeof(double));
  });
}

// Reduced-system build: kept mask, reduced rhs and Jacobi inverse diagonal
// scattered to full-length arrays, prescribed field (matfree.cpp:670-834).
int ref_build_reduced(int nx, int ny, int nz, double h, const uint8_t* solid,
                      const double* factor, double E, double nu, int nbc, const int* bc_node,
                      const int* bc_comp, const double* bc_val, int nload, const int* ld_node,
                      const int* ld_comp, const double* ld_val, uint8_t* kept, double* rhs,
                      double* invdiag, double* up, int* ng_out) {
  return guarded([&] {
    const VoxelGrid g = make_grid(nx, ny, nz, h, solid);
    std::vector<double> fv;
    if (factor) fv.assign(factor, factor + g.voxel_count());
    CgInfo info;
    const fea_detail::MatfreeReduced m = fea_detail::mf_build_reduced(
        g, E, nu, make_bcs(nbc, bc_node, bc_comp, bc_val),
        make_loads(nload, ld_node, ld_comp, ld_val), factor ? &fv : nullptr, "ref_build_reduced",
        &info);
    const std::size_t ndof = static_cast<std::size_t>(m.ndof);
    std::memset(kept, 0, ndof);
    std::memset(rhs, 0, ndof * sizeof(double));
    std::memset(invdiag, 0, ndof * sizeof(double));
    for (int k = 0; k < m.ng; ++k) {
      const int d = m.kept_global[static_cast<std::size_t>(k)];
      kept[d] = 1;
      rhs[d] = m.rg[static_cast<std::size_t>(k)];
      invdiag[d] = m.invdiag[static_cast<std::size_t>(k)];
    }
    std::memcpy(up, m.up.data(), ndof * sizeof(double));
    *ng_out = m.ng;
  });
}

// The reference's exact matrix-free Jacobi-PCG (fea_solve_cg_matfree).
int ref_solve_cg(int nx, int ny, int nz, double h, const uint8_t* solid, const double* factor,
                 double E, double nu, int nbc, const int* bc_node, const int* bc_comp,
                 const double* bc_val, int nload, const int* ld_node, const int* ld_comp,
                 const double* ld_val, double tol, int max_it, const double* initial_guess,
                 double* u, int* iters, double* resid) {
  CgInfo info;
  const int st = guarded([&] {
    const VoxelGrid g = make_grid(nx, ny, nz, h, solid);
    const auto bcs = make_bcs(nbc, bc_node, bc_comp, bc_val);
    const auto loads = make_loads(nload, ld_node, ld_comp, ld_val);
    FeaSolution sol;
    if (factor) {
      std::vector<double> fv(factor, factor + g.voxel_count());
      FeaSolution guess;
      if (initial_guess)
        guess.u.assign(initial_guess, initial_guess + 3 * static_cast<std::size_t>(fea_node_count(g)));
      sol = fea_solve_cg_matfree(g, fv, nu, bcs, loads, tol, max_it, &info,
                                 initial_guess ? &guess : nullptr, nullptr);
    } else {
      sol = fea_solve_cg_matfree(g, E, nu, bcs, loads, tol, max_it, &info);
    }
    std::memcpy(u, sol.u.data(), sol.u.size() * sizeof(double));
  });
  *iters = info.iterations;
  *resid = info.residual;
  return st;
}

// simp_compliance on the production solver kind; the oracle build routes its
// multigrid solve to the exact Jacobi-PCG (ref_shim.cpp).
int ref_simp_compliance(int nx, int ny, int nz, double h, const uint8_t* solid, double E0,
                        double nu, double penal, double rho_min, const double* density, int nbc,
                        const int* bc_node, const int* bc_comp, const double* bc_val, int nload,
                        const int* ld_node, const int* ld_comp, const double* ld_val, double tol,
                        int max_it, double* u, double* dc, double* compliance, int* iters,
                        double* resid) {
  return guarded([&] {
    const VoxelGrid g = make_grid(nx, ny, nz, h, solid);
    SimpParams p;
    p.youngs_modulus = E0;
    p.poisson = nu;
    p.penalty = penal;
    p.density_min = rho_min;
    std::vector<double> rho(density, density + g.voxel_count());
    const SimpCompliance c =
        simp_compliance(g, p, rho, make_bcs(nbc, bc_node, bc_comp, bc_val),
                        make_loads(nload, ld_node, ld_comp, ld_val), tol, max_it, nullptr,
                        nullptr, SolverKind::MultigridCG_Matfree);
    std::memcpy(u, c.solution.u.data(), c.solution.u.size() * sizeof(double));
    std::memcpy(dc, c.dcompliance.data(), c.dcompliance.size() * sizeof(double));
    *compliance = c.compliance;
    *iters = c.cg.iterations;
    *resid = c.cg.residual;
  });
}

int ref_filter(int nx, int ny, int nz, const uint8_t* solid, double radius, int adjoint,
               const double* x, double* out, double* weight_sum) {
  return guarded([&] {
    const VoxelGrid g = make_grid(nx, ny, nz, 1.0, solid);
    const DensityFilter f = make_density_filter(g, radius);
    std::vector<double> xv(x, x + g.voxel_count());
    const std::vector<double> o = adjoint ? f.filter_sensitivity(xv) : f.filter_density(xv);
    std::memcpy(out, o.data(), o.size() * sizeof(double));
    if (weight_sum) std::memcpy(weight_sum, f.weight_sum.data(), o.size() * sizeof(double));
  });
}

int ref_oc_update(int nx, int ny, int nz, const uint8_t* solid, double radius,
                  const double* density, const double* dc, double volfrac, double move,
                  double rho_min, double* x_new) {
  return guarded([&] {
    const VoxelGrid g = make_grid(nx, ny, nz, 1.0, solid);
    const DensityFilter f = make_density_filter(g, radius);
    std::vector<double> xv(density, density + g.voxel_count());
    std::vector<double> dv(dc, dc + g.voxel_count());
    const std::vector<double> o = oc_update(g, f, xv, dv, volfrac, move, rho_min);
    std::memcpy(x_new, o.data(), o.size() * sizeof(double));
  });
}

// simp_optimize with OC, no projection, SolverKind::MultigridCG_Matfree.
int ref_simp_optimize(int nx, int ny, int nz, double h, const uint8_t* solid, double E0,
                      double nu, double penal, double rho_min, int nbc, const int* bc_node,
                      const int* bc_comp, const double* bc_val, int nload, const int* ld_node,
                      const int* ld_comp, const double* ld_val, double volfrac, double radius,
                      double move, int max_it, double change_tol, double cg_tol, int cg_max_it,
                      double* hist_c, double* hist_change, double* hist_vf, double* design,
                      double* phys, double* out_scalars /* compliance, vf, init_c */,
                      int* out_ints /* iterations, converged, non_convergent, infeasible */) {
  return guarded([&] {
    const VoxelGrid g = make_grid(nx, ny, nz, h, solid);
    SimpParams p;
    p.youngs_modulus = E0;
    p.poisson = nu;
    p.penalty = penal;
    p.density_min = rho_min;
    SimpOptions o;
    o.volume_fraction = volfrac;
    o.filter_radius = radius;
    o.move = move;
    o.max_iterations = max_it;
    o.change_tol = change_tol;
    o.cg_tolerance = cg_tol;
    o.cg_max_iterations = cg_max_it;
    o.solver = SolverKind::MultigridCG_Matfree;
    const SimpOptimizeResult r = simp_optimize(g, p, make_bcs(nbc, bc_node, bc_comp, bc_val),
                                               make_loads(nload, ld_node, ld_comp, ld_val), o);
    for (std::size_t i = 0; i < r.history.size(); ++i) {
      hist_c[i] = r.history[i].compliance;
      hist_change[i] = r.history[i].change;
      hist_vf[i] = r.history[i].volume_fraction;
    }
    std::memcpy(design, r.design.data(), r.design.size() * sizeof(double));
    std::memcpy(phys, r.physical_density.data(), r.physical_density.size() * sizeof(double));
    out_scalars[0] = r.compliance;
    out_scalars[1] = r.volume_fraction;
    out_scalars[2] = r.initial_compliance;
    out_ints[0] = r.iterations;
    out_ints[1] = r.converged ? 1 : 0;
    out_ints[2] = r.non_convergent ? 1 : 0;
    out_ints[3] = r.infeasible ? 1 : 0;
  });
}

int ref_effective_design_mask(int nx, int ny, int nz, const uint8_t* tags, const uint8_t* mask,
                              uint8_t* eff) {
  return guarded([&] {
    const VoxelGrid g = make_grid_tags(nx, ny, nz, 1.0, tags);
    const DesignMask m = effective_design_mask(g, make_mask(g.voxel_count(), mask));
    for (std::size_t e = 0; e < m.size(); ++e) eff[e] = static_cast<uint8_t>(m[e]);
  });
}

// make_density_filter(grid, radius, mask) with raw tags and a caller mask.
int ref_filter_masked(int nx, int ny, int nz, const uint8_t* tags, const uint8_t* mask,
                      double radius, int adjoint, const double* x, double* out) {
  return guarded([&] {
    const VoxelGrid g = make_grid_tags(nx, ny, nz, 1.0, tags);
    const DensityFilter f = make_density_filter(g, radius, make_mask(g.voxel_count(), mask));
    std::vector<double> xv(x, x + g.voxel_count());
    const std::vector<double> o = adjoint ? f.filter_sensitivity(xv) : f.filter_density(xv);
    std::memcpy(out, o.data(), o.size() * sizeof(double));
  });
}

// The masked simp_optimize overload (OC, no projection, MultigridCG_Matfree).
int ref_simp_optimize_masked(int nx, int ny, int nz, double h, const uint8_t* tags,
                             const uint8_t* mask, double E0, double nu, double penal,
                             double rho_min, int nbc, const int* bc_node, const int* bc_comp,
                             const double* bc_val, int nload, const int* ld_node,
                             const int* ld_comp, const double* ld_val, double volfrac,
                             double radius, double move, int max_it, double change_tol,
                             double cg_tol, int cg_max_it, double* hist_c, double* hist_change,
                             double* hist_vf, double* design, double* phys,
                             double* out_scalars, int* out_ints) {
  return guarded([&] {
    const VoxelGrid g = make_grid_tags(nx, ny, nz, h, tags);
    SimpParams p;
    p.youngs_modulus = E0;
    p.poisson = nu;
    p.penalty = penal;
    p.density_min = rho_min;
    SimpOptions o;
    o.volume_fraction = volfrac;
    o.filter_radius = radius;
    o.move = move;
    o.max_iterations = max_it;
    o.change_tol = change_tol;
    o.cg_tolerance = cg_tol;
    o.cg_max_iterations = cg_max_it;
    o.solver = SolverKind::MultigridCG_Matfree;
    const SimpOptimizeResult r =
        simp_optimize(g, p, make_bcs(nbc, bc_node, bc_comp, bc_val),
                      make_loads(nload, ld_node, ld_comp, ld_val), o,
                      make_mask(g.voxel_count(), mask));
    for (std::size_t i = 0; i < r.history.size(); ++i) {
      hist_c[i] = r.history[i].compliance;
      hist_change[i] = r.history[i].change;
      hist_vf[i] = r.history[i].volume_fraction;
    }
    std::memcpy(design, r.design.data(), r.design.size() * sizeof(double));
    std::memcpy(phys, r.physical_density.data(), r.physical_density.size() * sizeof(double));
    out_scalars[0] = r.compliance;
    out_scalars[1] = r.volume_fraction;
    out_scalars[2] = r.initial_compliance;
    out_ints[0] = r.iterations;
    out_ints[1] = r.converged ? 1 : 0;
    out_ints[2] = r.non_convergent ? 1 : 0;
    out_ints[3] = r.infeasible ? 1 : 0;
  });
}

int ref_project(double rt, double beta, double eta, double* value, double* derivative) {
  return guarded([&] {
    *value = heaviside_project(rt, beta, eta);
    *derivative = heaviside_project_derivative(rt, beta, eta);
  });
}

// simp_optimize with OC and a Heaviside projection schedule (the projected
// formulation of simp.cpp:2018-2592), MultigridCG_Matfree.
int ref_simp_optimize_projected(int nx, int ny, int nz, double h, const uint8_t* solid, double E0,
                                double nu, double penal, double rho_min, int nbc,
                                const int* bc_node, const int* bc_comp, const double* bc_val,
                                int nload, const int* ld_node, const int* ld_comp,
                                const double* ld_val, double volfrac, double radius,
                                double change_tol, double cg_tol, int cg_max_it, int nstages,
                                const double* beta, const double* move, const int* iters,
                                double eta, double* hist_c, double* hist_change, double* hist_vf,
                                double* design, double* phys, double* out_scalars,
                                int* out_ints) {
  return guarded([&] {
    const VoxelGrid g = make_grid(nx, ny, nz, h, solid);
    SimpParams p;
    p.youngs_modulus = E0;
    p.poisson = nu;
    p.penalty = penal;
    p.density_min = rho_min;
    SimpOptions o;
    o.volume_fraction = volfrac;
    o.filter_radius = radius;
    o.change_tol = change_tol;
    o.cg_tolerance = cg_tol;
    o.cg_max_iterations = cg_max_it;
    o.solver = SolverKind::MultigridCG_Matfree;
    o.projection_eta = eta;
    for (int k = 0; k < nstages; ++k) {
      ProjectionStage ps;
      ps.beta = beta[k];
      ps.move = move[k];
      ps.iterations = iters[k];
      o.projection.push_back(ps);
    }
    const SimpOptimizeResult r = simp_optimize(g, p, make_bcs(nbc, bc_node, bc_comp, bc_val),
                                               make_loads(nload, ld_node, ld_comp, ld_val), o);
    for (std::size_t i = 0; i < r.history.size(); ++i) {
      hist_c[i] = r.history[i].compliance;
      hist_change[i] = r.history[i].change;
      hist_vf[i] = r.history[i].volume_fraction;
    }
    std::memcpy(design, r.design.data(), r.design.size() * sizeof(double));
    std::memcpy(phys, r.physical_density.data(), r.physical_density.size() * sizeof(double));
    out_scalars[0] = r.compliance;
    out_scalars[1] = r.volume_fraction;
    out_scalars[2] = r.initial_compliance;
    out_ints[0] = r.iterations;
    out_ints[1] = r.converged ? 1 : 0;
    out_ints[2] = r.non_convergent ? 1 : 0;
    out_ints[3] = r.infeasible ? 1 : 0;
  });
}


// hex8_stress (hex_element.cpp:242-316).
int ref_hex8_stress(double E, double nu, double h, const double* ue, double xi, double eta,
                    double zeta, double* sigma6, double* von_mises) {
  return guarded([&] {
    std::array<double, 24> u{};
    for (int q = 0; q < 24; ++q) u[static_cast<std::size_t>(q)] = ue[q];
    const Hex8Stress st = hex8_stress(E, nu, h, u, xi, eta, zeta);
    for (int r = 0; r < 6; ++r) sigma6[r] = st.sigma[static_cast<std::size_t>(r)];
    *von_mises = st.von_mises;
  });
}

// compute_stress_margin (settings/report.cpp:464-491).
int ref_stress_margin(double yield, double zk, double vm, double il, double* out3) {
  return guarded([&] {
    const StressMargin m = compute_stress_margin(yield, zk, vm, il);
    out3[0] = m.in_plane;
    out3[1] = m.interlayer;
    out3[2] = m.worst_case;
  });
}

// load_path_connected (voxelize.cpp:609-726).
int ref_load_path_connected(int nx, int ny, int nz, const uint8_t* tags, const double* density,
                            double iso, int* out) {
  return guarded([&] {
    const VoxelGrid g = make_grid_tags(nx, ny, nz, 1.0, tags);
    *out = load_path_connected(g, std::vector<double>(density, density + g.voxel_count()), iso)
               ? 1
               : 0;
  });
}

// The solid-posture core of analyze_fixed_design (analyze.cpp:145-440) from the
// reference's own pieces: simp_compliance at cg_tol with the matrix-free
// multigrid, hex8_stress at every printed voxel's centre with the solid modulus,
// max_interlayer_tension, compute_stress_margin, load_path_connected.
// out_d = {compliance, max_vm, max_il, in_plane, interlayer, worst, effective};
// out_i = {non_convergent, printed_voxels, load_path_ok, accepted}.
namespace {
void ref_analysis(const VoxelGrid& g, const SimpParams& p, const std::vector<double>& rho,
                  const std::vector<DirichletBC>& bcs, const std::vector<NodalLoad>& loads,
                  double yield, double zk, const double* bdir, double iso, double knock,
                  double margin_stop, double cg_tol, int cg_max_it, double* out_d, int* out_i,
                  double* vm_field) {
  for (int q = 0; q < 7; ++q) out_d[q] = 0.0;
  for (int q = 0; q < 4; ++q) out_i[q] = 0;
  SimpCompliance sc;
  try {
    sc = simp_compliance(g, p, rho, bcs, loads, cg_tol, cg_max_it, nullptr, nullptr,
                         SolverKind::MultigridCG_Matfree);
  } catch (const SolverNonConvergence&) {
    out_i[0] = 1;
    return;
  }
  out_d[0] = sc.compliance;
  std::vector<std::array<double, 6>> stress(g.voxel_count(), std::array<double, 6>{});
  double max_vm = 0.0;
  int printed = 0;
  for (int k = 0; k < g.nz; ++k)
    for (int j = 0; j < g.ny; ++j)
      for (int i = 0; i < g.nx; ++i) {
        if (!g.solid(i, j, k)) continue;
        const std::size_t idx = g.index(i, j, k);
        if (!(rho[idx] > iso)) continue;
        ++printed;
        const std::array<int, 8> en = fea_element_nodes(g, i, j, k);
        std::array<double, 24> ue{};
        for (int a = 0; a < 8; ++a)
          for (int c = 0; c < 3; ++c)
            ue[static_cast<std::size_t>(3 * a + c)] = sc.solution.at(en[static_cast<std::size_t>(a)], c);
        const Hex8Stress st = hex8_stress(p.youngs_modulus, p.poisson, g.spacing, ue);
        stress[idx] = st.sigma;
        if (vm_field) vm_field[idx] = st.von_mises;
        if (st.von_mises > max_vm) max_vm = st.von_mises;
      }
  const double max_il = max_interlayer_tension(g, stress, Vec3{bdir[0], bdir[1], bdir[2]});
  const StressMargin m = compute_stress_margin(yield, zk, max_vm, max_il);
  out_d[1] = max_vm;
  out_d[2] = max_il;
  out_d[3] = m.in_plane;
  out_d[4] = m.interlayer;
  out_d[5] = m.worst_case;
  out_d[6] = m.worst_case * knock;
  out_i[1] = printed;
  out_i[2] = load_path_connected(g, rho, iso) ? 1 : 0;
  out_i[3] = (out_i[2] && out_d[6] >= margin_stop) ? 1 : 0;
}
}  // namespace

int ref_analyze_fixed_design(int nx, int ny, int nz, double h, const uint8_t* tags, double E0,
                             double nu, double penal, double rho_min, const double* density,
                             int nbc, const int* bc_node, const int* bc_comp,
                             const double* bc_val, int nload, const int* ld_node,
                             const int* ld_comp, const double* ld_val, double yield, double zk,
                             const double* bdir, double iso, double knock, double margin_stop,
                             double cg_tol, int cg_max_it, double* out_d, int* out_i,
                             double* vm_field) {
  return guarded([&] {
    const VoxelGrid g = make_grid_tags(nx, ny, nz, h, tags);
    SimpParams p;
    p.youngs_modulus = E0;
    p.poisson = nu;
    p.penalty = penal;
    p.density_min = rho_min;
    ref_analysis(g, p, std::vector<double>(density, density + g.voxel_count()),
                 make_bcs(nbc, bc_node, bc_comp, bc_val), make_loads(nload, ld_node, ld_comp, ld_val),
                 yield, zk, bdir, iso, knock, margin_stop, cg_tol, cg_max_it, out_d, out_i,
                 vm_field);
  });
}

// The ladder walk of minimize_plastic (minimize_plastic.cpp:1402-2742) for the
// OC updater, driven through the reference's own simp_optimize (masked
// overload, SimpOptions::initial_design as the warm seed) and the analysis
// above.  Per rung r: rung_d[8r..] = {vf, compliance, max_vm, max_il, worst,
// effective, 0, 0}, rung_i[6r..] = {iterations, trajectory_ok, analysed,
// accepted, load_path_ok, non_convergent_analysis}.  out_i = {evaluated,
// recommended, stopped_on_margin}.
int ref_ladder(int nx, int ny, int nz, double h, const uint8_t* tags, const uint8_t* mask,
               double E0, double nu, double penal, double rho_min, int nbc, const int* bc_node,
               const int* bc_comp, const double* bc_val, int nload, const int* ld_node,
               const int* ld_comp, const double* ld_val, double radius, double move, int max_it,
               double change_tol, double cg_tol, int cg_max_it, const double* ladder, int nrungs,
               int inherit, double yield, double zk, const double* bdir, double iso,
               double knock, double margin_stop, double* rung_d, int* rung_i, int* out_i,
               double* design, double* phys) {
  return guarded([&] {
    const VoxelGrid g = make_grid_tags(nx, ny, nz, h, tags);
    const std::size_t nv = g.voxel_count();
    SimpParams p;
    p.youngs_modulus = E0;
    p.poisson = nu;
    p.penalty = penal;
    p.density_min = rho_min;
    const auto bcs = make_bcs(nbc, bc_node, bc_comp, bc_val);
    const auto loads = make_loads(nload, ld_node, ld_comp, ld_val);
    std::vector<uint8_t> zeros;
    if (!mask) {
      zeros.assign(nv, 0);
      mask = zeros.data();
    }
    const DesignMask dm = make_mask(nv, mask);
    std::vector<double> seed;
    out_i[0] = 0;
    out_i[1] = -1;
    out_i[2] = 0;
    for (int r = 0; r < nrungs; ++r) {
      SimpOptions o;
      o.volume_fraction = ladder[r];
      o.filter_radius = radius;
      o.move = move;
      o.max_iterations = max_it;
      o.change_tol = change_tol;
      o.cg_tolerance = cg_tol;
      o.cg_max_iterations = cg_max_it;
      o.solver = SolverKind::MultigridCG_Matfree;
      o.initial_design = seed;
      const SimpOptimizeResult res = simp_optimize(g, p, bcs, loads, o, dm);
      double* d = rung_d + 8 * r;
      int* ii = rung_i + 6 * r;
      for (int q = 0; q < 8; ++q) d[q] = 0.0;
      for (int q = 0; q < 6; ++q) ii[q] = 0;
      d[0] = ladder[r];
      d[1] = res.compliance;
      ii[0] = res.iterations;
      out_i[0] = r + 1;
      if (res.infeasible || res.non_convergent) continue;
      ii[1] = 1;
      const std::vector<double>& rho = res.physical_density;
      if (load_path_connected(g, rho, iso)) seed = inherit ? rho : std::vector<double>();
      double ad[7];
      int ai[4];
      ref_analysis(g, p, rho, bcs, loads, yield, zk, bdir, iso, knock, margin_stop, cg_tol,
                   cg_max_it, ad, ai, nullptr);
      d[2] = ad[1];
      d[3] = ad[2];
      d[4] = ad[5];
      d[5] = ad[6];
      ii[4] = ai[2];
      ii[5] = ai[0];
      if (ai[0]) continue;
      ii[2] = 1;
      ii[3] = ai[3];
      if (ai[3]) {
        out_i[1] = r;
        if (design) std::memcpy(design, res.design.data(), nv * sizeof(double));
        if (phys) std::memcpy(phys, rho.data(), nv * sizeof(double));
      } else if (!(ad[6] >= margin_stop)) {
        out_i[2] = 1;
        break;
      }
    }
  });
}


// The reference's own writers of design.bin (design_store.cpp), fields.bin
// (fields.cpp) and one iterations.csv row (IterationCsvWriter::append_at), fed
// variants built from flat arrays.  Per design variant: d = {requested vf,
// achieved vf, worst, effective, max vm, dir x, y, z}, i = {accepted,
// iterations, auto applied, export baked}.
int ref_write_design_file(const char* path, int nx, int ny, int nz, const double* origin,
                          double spacing, int nvar, const double* d, const int* ii,
                          const double* dens) {
  return guarded([&] {
    VoxelGrid g = make_grid(nx, ny, nz, spacing, nullptr);
    g.origin = Vec3{origin[0], origin[1], origin[2]};
    const std::size_t nv = g.voxel_count();
    std::vector<MinimizePlasticVariant> vs(static_cast<std::size_t>(nvar));
    std::vector<const MinimizePlasticVariant*> ptrs;
    for (int k = 0; k < nvar; ++k) {
      MinimizePlasticVariant& v = vs[static_cast<std::size_t>(k)];
      const double* dk = d + 8 * k;
      const int* ik = ii + 4 * k;
      v.requested_volume_fraction = dk[0];
      v.optimization.volume_fraction = dk[1];
      v.report.margin.worst_case = dk[2];
      v.report.margin_effective = dk[3];
      v.report.max_stress_mpa = dk[4];
      v.applied_build_dir = Vec3{dk[5], dk[6], dk[7]};
      v.accepted = ik[0] != 0;
      v.optimization.iterations = ik[1];
      v.build_direction_auto_applied = ik[2] != 0;
      v.export_baked = ik[3] != 0;
      v.optimization.physical_density.assign(dens + std::size_t(k) * nv,
                                             dens + std::size_t(k + 1) * nv);
      ptrs.push_back(&v);
    }
    write_design_file(path, ptrs, g);
  });
}

uint64_t ref_design_fingerprint(const double* d, long long n) {
  return design_fingerprint(std::vector<double>(d, d + n));
}

// fields.bin: per variant d = {requested vf, mass}, i = {support voxels}.
int ref_write_fields_file(const char* path, int nx, int ny, int nz, const double* origin,
                          double spacing, int nvar, const double* d, const int* ii,
                          const double* vm, const double* disp) {
  return guarded([&] {
    VoxelGrid g = make_grid(nx, ny, nz, spacing, nullptr);
    g.origin = Vec3{origin[0], origin[1], origin[2]};
    const std::size_t nv = g.voxel_count();
    const std::size_t nd = 3 * std::size_t(fea_node_count(g));
    std::vector<MinimizePlasticVariant> vs(static_cast<std::size_t>(nvar));
    std::vector<const MinimizePlasticVariant*> ptrs;
    for (int k = 0; k < nvar; ++k) {
      MinimizePlasticVariant& v = vs[static_cast<std::size_t>(k)];
      v.accepted = true;
      v.requested_volume_fraction = d[2 * k];
      v.mass_grams = d[2 * k + 1];
      v.support_volume_voxels = ii[k];
      v.von_mises_field.assign(vm + std::size_t(k) * nv, vm + std::size_t(k + 1) * nv);
      v.displacement_field.assign(disp + std::size_t(k) * nd, disp + std::size_t(k + 1) * nd);
      ptrs.push_back(&v);
    }
    write_fields_file(path, ptrs, g);
  });
}

// One iterations.csv (header + one row) from an observation given as flat
// arrays: od = {compliance, volume_fraction, beta, active_fraction, 18 phase
// times in schema order, rss, peak_rss, compressed, available}; oi =
// {iteration, plateau, cg_iters, cg_multigrid, hier_built, mg_cycles,
// infeasible, recycle_dim, geneo_dim, geneo_action, geneo_burn,
// geneo_threshold}; ol = {fea_solves, matvecs, major_faults, swapins}.
int ref_iteration_csv(const char* path, long long rung, const double* od, const int* oi,
                      const long long* ol, long long wall_ms) {
  return guarded([&] {
    SimpIterationObservation o;
    o.compliance = od[0];
    o.volume_fraction = od[1];
    o.beta = od[2];
    o.active_fraction = od[3];
    double* ph[18] = {&o.phases.total_ms, &o.phases.tail_prev_ms, &o.phases.filter_ms,
                      &o.phases.project_ms, &o.phases.solve_ms, &o.phases.fea_ms,
                      &o.phases.sens_ms, &o.phases.update_ms, &o.phases.analysis_ms,
                      &o.phases.observe_ms, &o.phases.residual_ms, &o.phases.solver_build_ms,
                      &o.phases.solver_mg_build_ms, &o.phases.solver_mg_ms,
                      &o.phases.solver_cg_ms, &o.phases.solver_geneo_setup_ms,
                      &o.phases.solver_geneo_apply_ms, &o.phases.solver_recycle_ms};
    for (int q = 0; q < 18; ++q) *ph[q] = od[4 + q];
    o.phases.rss_mb = od[22];
    o.phases.peak_rss_mb = od[23];
    o.phases.compressed_mb = od[24];
    o.phases.available_mb = od[25];
    o.iteration = oi[0];
    o.plateau = oi[1] != 0;
    o.cg_iterations = oi[2];
    o.cg_used_multigrid = oi[3] != 0;
    o.cg_hier_built = oi[4] != 0;
    o.cg_mg_cycles_attempted = oi[5];
    o.infeasible = oi[6] != 0;
    o.cg_recycle_dim = oi[7];
    o.cg_geneo_dim = oi[8];
    o.cg_geneo_action = oi[9];
    o.cg_geneo_burn = oi[10];
    o.cg_geneo_threshold = oi[11];
    o.phases.fea_solves = ol[0];
    o.phases.matvecs = ol[1];
    o.phases.major_faults = ol[2];
    o.phases.swapins = ol[3];
    IterationCsvWriter w(path);
    w.append_at(static_cast<std::size_t>(rung), o, wall_ms);
  });
}

// simp_optimize with the MMA updater (SimpUpdater::MMA, simp.cpp:2305-2311 and
// the masked :3350-3357), plain when mask is NULL, MultigridCG_Matfree, with the
// plateau options mma_plateau_{window, tol, min_drop, flat_windows}.
int ref_simp_optimize_mma(int nx, int ny, int nz, double h, const uint8_t* tags,
                          const uint8_t* mask, double E0, double nu, double penal,
                          double rho_min, int nbc, const int* bc_node, const int* bc_comp,
                          const double* bc_val, int nload, const int* ld_node,
                          const int* ld_comp, const double* ld_val, double volfrac,
                          double radius, double move, int max_it, double change_tol,
                          double cg_tol, int cg_max_it, int pw, double ptol, double pdrop,
                          int pflat, double* hist_c, double* hist_change, double* hist_vf,
                          double* design, double* phys, double* out_scalars, int* out_ints) {
  return guarded([&] {
    const VoxelGrid g = make_grid_tags(nx, ny, nz, h, tags);
    SimpParams p;
    p.youngs_modulus = E0;
    p.poisson = nu;
    p.penalty = penal;
    p.density_min = rho_min;
    SimpOptions o;
    o.volume_fraction = volfrac;
    o.filter_radius = radius;
    o.move = move;
    o.max_iterations = max_it;
    o.change_tol = change_tol;
    o.cg_tolerance = cg_tol;
    o.cg_max_iterations = cg_max_it;
    o.solver = SolverKind::MultigridCG_Matfree;
    o.updater = SimpUpdater::MMA;
    o.mma_plateau_window = pw;
    o.mma_plateau_tol = ptol;
    o.mma_plateau_min_drop = pdrop;
    o.mma_plateau_flat_windows = pflat;
    const auto bcs = make_bcs(nbc, bc_node, bc_comp, bc_val);
    const auto loads = make_loads(nload, ld_node, ld_comp, ld_val);
    const SimpOptimizeResult r =
        mask ? simp_optimize(g, p, bcs, loads, o, make_mask(g.voxel_count(), mask))
             : simp_optimize(g, p, bcs, loads, o);
    for (std::size_t i = 0; i < r.history.size(); ++i) {
      hist_c[i] = r.history[i].compliance;
      hist_change[i] = r.history[i].change;
      hist_vf[i] = r.history[i].volume_fraction;
    }
    std::memcpy(design, r.design.data(), r.design.size() * sizeof(double));
    std::memcpy(phys, r.physical_density.data(), r.physical_density.size() * sizeof(double));
    out_scalars[0] = r.compliance;
    out_scalars[1] = r.volume_fraction;
    out_scalars[2] = r.initial_compliance;
    out_ints[0] = r.iterations;
    out_ints[1] = r.converged ? 1 : 0;
    out_ints[2] = r.non_convergent ? 1 : 0;
    out_ints[3] = r.infeasible ? 1 : 0;
  });
}

// active_domain_auto_band / active_domain_mask / active_domain_escape_count.
int ref_active_domain_auto_band(double radius) { return active_domain_auto_band(radius); }

int ref_active_domain_mask(int nx, int ny, int nz, const uint8_t* tags, const double* density,
                           double rho_min, int band, uint8_t* out) {
  return guarded([&] {
    const VoxelGrid g = make_grid_tags(nx, ny, nz, 1.0, tags);
    const std::vector<double> d(density, density + g.voxel_count());
    const std::vector<char> m = active_domain_mask(g, d, rho_min, band);
    for (std::size_t e = 0; e < m.size(); ++e) out[e] = static_cast<uint8_t>(m[e]);
  });
}

int ref_active_domain_escape_count(int nx, int ny, int nz, const uint8_t* tags,
                                   const double* density, const uint8_t* prev, double rho_min,
                                   long long* out) {
  return guarded([&] {
    const VoxelGrid g = make_grid_tags(nx, ny, nz, 1.0, tags);
    const std::vector<double> d(density, density + g.voxel_count());
    std::vector<char> pm;
    if (prev) pm.assign(prev, prev + g.voxel_count());
    *out = active_domain_escape_count(g, d, pm, rho_min);
  });
}

// simp_optimize (OC, or MMA with updater 1; MultigridCG_Matfree; plain when
// mask is NULL) with options.active_domain_band = band and an optional
// warm-start seed; the
// per-iteration active fraction comes from the observe hook.
// out_ints: iterations, converged, non_convergent, infeasible, band, latched,
// latch_iteration, escape_count.  out_scalars: compliance, vf, init_c,
// active_fraction_mean.  reason: 256 bytes.
int ref_simp_optimize_active(int nx, int ny, int nz, double h, const uint8_t* tags,
                             const uint8_t* mask, double E0, double nu, double penal,
                             double rho_min, int nbc, const int* bc_node, const int* bc_comp,
                             const double* bc_val, int nload, const int* ld_node,
                             const int* ld_comp, const double* ld_val, double volfrac,
                             double radius, double move, int max_it, double change_tol,
                             double cg_tol, int cg_max_it, int band, int updater,
                             const double* seed,
                             double* hist_c, double* hist_change, double* hist_vf,
                             double* hist_af, double* design, double* phys,
                             double* out_scalars, long long* out_ints, char* reason) {
  return guarded([&] {
    const VoxelGrid g = make_grid_tags(nx, ny, nz, h, tags);
    SimpParams p;
    p.youngs_modulus = E0;
    p.poisson = nu;
    p.penalty = penal;
    p.density_min = rho_min;
    SimpOptions o;
    o.volume_fraction = volfrac;
    o.filter_radius = radius;
    o.move = move;
    o.max_iterations = max_it;
    o.change_tol = change_tol;
    o.cg_tolerance = cg_tol;
    o.cg_max_iterations = cg_max_it;
    o.solver = SolverKind::MultigridCG_Matfree;
    o.active_domain_band = band;
    if (updater == 1) o.updater = SimpUpdater::MMA;  // plateau stop at its defaults
    if (seed) o.initial_design.assign(seed, seed + g.voxel_count());
    std::vector<double> af;
    o.observe = [&](const SimpIterationObservation& ob) { af.push_back(ob.active_fraction); };
    const auto bcs = make_bcs(nbc, bc_node, bc_comp, bc_val);
    const auto loads = make_loads(nload, ld_node, ld_comp, ld_val);
    const SimpOptimizeResult r =
        mask ? simp_optimize(g, p, bcs, loads, o, make_mask(g.voxel_count(), mask))
             : simp_optimize(g, p, bcs, loads, o);
    for (std::size_t i = 0; i < r.history.size(); ++i) {
      hist_c[i] = r.history[i].compliance;
      hist_change[i] = r.history[i].change;
      hist_vf[i] = r.history[i].volume_fraction;
    }
    for (std::size_t i = 0; i < af.size(); ++i) hist_af[i] = af[i];
    std::memcpy(design, r.design.data(), r.design.size() * sizeof(double));
    std::memcpy(phys, r.physical_density.data(), r.physical_density.size() * sizeof(double));
    out_scalars[0] = r.compliance;
    out_scalars[1] = r.volume_fraction;
    out_scalars[2] = r.initial_compliance;
    out_scalars[3] = r.active_fraction_mean;
    out_ints[0] = r.iterations;
    out_ints[1] = r.converged ? 1 : 0;
    out_ints[2] = r.non_convergent ? 1 : 0;
    out_ints[3] = r.infeasible ? 1 : 0;
    out_ints[4] = r.active_domain_band;
    out_ints[5] = r.active_domain_latched ? 1 : 0;
    out_ints[6] = r.active_domain_latch_iteration;
    out_ints[7] = r.active_domain_escape_count;
    std::memset(reason, 0, 256);
    std::strncpy(reason, r.active_domain_latch_reason.c_str(), 255);
  });
}
}  // extern "C"
