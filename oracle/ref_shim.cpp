// ref_shim.cpp -- closes the 31 symbols the reference's Eigen-free translation
// units leave unresolved, so its own hot-path code (hex_element.cpp, matfree.cpp,
// recycle.cpp, simp.cpp and their base files) links into oracle/_ref/.
//
// TEST INFRASTRUCTURE ONLY: linked into the reference build that the tests and
// the CPU baseline use as a checker; never into the product library.
//
//  * fea_node_count / fea_node_index / fea_element_nodes: the three formulas of
//    core/include/topopt/fea.hpp:140-157 (their definitions live in
//    core/src/fea/assembly.cpp, which needs Eigen).
//  * fea_detail::geneo_*: GenEO is library-default OFF (fea.hpp:1022); the stubs
//    report "disabled", which keeps mf_cg_solve on its plain path.
//  * fea_solve_mgcg_matfree (graded): routed to the reference's own exact
//    matrix-free Jacobi-PCG, fea_solve_cg_matfree (matfree.cpp:1106), which solves
//    the identical reduced, void-gated system to the same relative-residual test.
//    CgInfo::used_multigrid stays false.
//  * Everything else (assembled / lattice solvers, PenalizedSolver) needs Eigen
//    and is unused on the MultigridCG_Matfree route (simp.cpp:2126-2128): they
//    throw std::logic_error if ever reached.
#include <stdexcept>

#include "fea/geneo.hpp"
#include "fea/fea_matfree.hpp"
#include "topopt/fea.hpp"

namespace topopt {

int fea_node_count(const VoxelGrid& grid) {
  return (grid.nx + 1) * (grid.ny + 1) * (grid.nz + 1);
}

int fea_node_index(const VoxelGrid& grid, int a, int b, int c) {
  return (c * (grid.ny + 1) + b) * (grid.nx + 1) + a;
}

std::array<int, 8> fea_element_nodes(const VoxelGrid& grid, int i, int j, int k) {
  return {fea_node_index(grid, i, j, k),         fea_node_index(grid, i + 1, j, k),
          fea_node_index(grid, i + 1, j + 1, k), fea_node_index(grid, i, j + 1, k),
          fea_node_index(grid, i, j, k + 1),     fea_node_index(grid, i + 1, j, k + 1),
          fea_node_index(grid, i + 1, j + 1, k + 1), fea_node_index(grid, i, j + 1, k + 1)};
}

[[noreturn]] static void unavailable(const char* who) {
  throw std::logic_error(std::string(who) + ": needs Eigen; not part of the oracle build");
}

FeaSolution fea_solve_cg(const VoxelGrid&, const std::vector<double>&, double,
                         const std::vector<DirichletBC>&, const std::vector<NodalLoad>&, double,
                         int, CgInfo*, const FeaSolution*) {
  unavailable("fea_solve_cg");
}
FeaSolution fea_solve_mgcg(const VoxelGrid&, const std::vector<double>&, double,
                           const std::vector<DirichletBC>&, const std::vector<NodalLoad>&,
                           double, int, CgInfo*) {
  unavailable("fea_solve_mgcg");
}
FeaSolution fea_solve_cg_lattice(const VoxelGrid&, const std::vector<double>&,
                                 const std::vector<char>&, const std::vector<double>&,
                                 const std::vector<double>&, const std::vector<double>&, double,
                                 const std::vector<DirichletBC>&, const std::vector<NodalLoad>&,
                                 double, int, CgInfo*) {
  unavailable("fea_solve_cg_lattice");
}
FeaSolution fea_solve_cg_lattice_matfree(const VoxelGrid&, const std::vector<double>&,
                                         const std::vector<char>&, const std::vector<double>&,
                                         const std::vector<double>&, const std::vector<double>&,
                                         double, const std::vector<DirichletBC>&,
                                         const std::vector<NodalLoad>&, double, int, CgInfo*,
                                         const std::vector<char>*) {
  unavailable("fea_solve_cg_lattice_matfree");
}

FeaSolution fea_solve_mgcg_matfree(const VoxelGrid& grid,
                                   const std::vector<double>& youngs_per_voxel, double poisson,
                                   const std::vector<DirichletBC>& bcs,
                                   const std::vector<NodalLoad>& loads, double tolerance,
                                   int max_iterations, CgInfo* info,
                                   const std::vector<char>* active_mask,
                                   const FeaSolution* initial_guess) {
  return fea_solve_cg_matfree(grid, youngs_per_voxel, poisson, bcs, loads, tolerance,
                              max_iterations, info, initial_guess, active_mask);
}

struct PenalizedSolver::Impl {};
PenalizedSolver::PenalizedSolver(const VoxelGrid&, double, const std::vector<DirichletBC>&,
                                 const std::vector<NodalLoad>&) {
  unavailable("PenalizedSolver");
}
PenalizedSolver::~PenalizedSolver() = default;
bool PenalizedSolver::usable() const { return false; }
FeaSolution PenalizedSolver::solve(const std::vector<double>&, double, int, CgInfo*) {
  unavailable("PenalizedSolver::solve");
}

namespace fea_detail {
bool geneo_enabled() { return false; }
bool geneo_set_enabled(bool) { return false; }
void geneo_reset() {}
void geneo_solve_begin(const MatfreeReduced&, const MfSolveContext&) {}
int geneo_engage_threshold() { return -1; }
bool geneo_engage_now(const MatfreeReduced&, const MfSolveContext&, int) { return false; }
void geneo_apply(const double*, double*) {}
void geneo_solve_end(int, bool) {}
GeneoReport geneo_last_report() { return GeneoReport{}; }
long long geneo_basis_builds() { return 0; }
long long geneo_coarse_refreshes() { return 0; }
long long geneo_armed_solves() { return 0; }
long long geneo_declined_solves() { return 0; }
int geneo_basis_dim() { return 0; }
std::size_t geneo_basis_bytes() { return 0; }
int geneo_decision_count() { return 0; }
GeneoDecision geneo_decision_at(int) { return GeneoDecision{}; }
long long geneo_decisions_dropped() { return 0; }
const GeneoProbeConfig& geneo_probe_config() {
  static const GeneoProbeConfig cfg{};
  return cfg;
}
}  // namespace fea_detail

}  // namespace topopt
