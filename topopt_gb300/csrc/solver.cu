// solver.cu -- host orchestration of the reduced system and its solvers.
//
// Reference counterparts:
//   mf_build_reduced (void-DOF gate)   core/src/fea/matfree.cpp:670-834
//   mf_cg_solve (Eigen-style Jacobi-PCG, the exact fallback) matfree.cpp:841-1076
//   build_mf_hierarchy / v_cycle / mf_mgpcg   core/src/fea/multigrid.cpp:1344-1515,
//                                             :780-817, :1143-1160, :1211-1313
//   solve_mgcg_matfree (budget, fallback)      multigrid.cpp:2098-2320
//   mixed-precision V-cycle (FP32 fine level)  multigrid.cpp:1179-1204
//
// Everything numeric runs on the device; the host only sequences launches and
// reads two or three FP64 scalars per Krylov iteration (the convergence test).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <limits>
#include <system_error>
#include <thread>

#include "tg_solver.h"

namespace tg {

namespace {
double now_ms() {
  return std::chrono::duration<double, std::milli>(
             std::chrono::steady_clock::now().time_since_epoch())
      .count();
}
// Hex8 local node order -> corner bit index (x | y<<1 | z<<2).
const int kLocToBit[8] = {0, 1, 3, 2, 4, 5, 7, 6};
const double kXi[8] = {-1, +1, +1, -1, -1, +1, +1, -1};
const double kEta[8] = {-1, -1, +1, +1, -1, -1, +1, +1};
const double kZeta[8] = {-1, -1, -1, -1, +1, +1, +1, +1};
constexpr int kMaxCoarseDof = 8192;   // dense coarsest factor <= 512 MB
constexpr int kMaxInverseDof = 512;   // explicit coarsest inverse up to here
constexpr int64_t kAutotuneMinVoxels = int64_t(1) << 20;  // FP32 schedule measured from here

MgDims dims_of(int ex, int ey, int ez) { return MgDims{ex, ey, ez, ex + 1, ey + 1, ez + 1}; }
}  // namespace

// 2x2x2 Gauss integration of B^T D B (the reference's quadrature,
// hex_element.cpp:23-89), isotropic D (:93-115).
void hex8_ke(double E, double nu, double h, double* ke) {
  double D[6][6] = {};
  const double c = E / ((1.0 + nu) * (1.0 - 2.0 * nu));
  D[0][0] = D[1][1] = D[2][2] = c * (1.0 - nu);
  D[0][1] = D[0][2] = D[1][0] = D[1][2] = D[2][0] = D[2][1] = c * nu;
  D[3][3] = D[4][4] = D[5][5] = c * (1.0 - 2.0 * nu) / 2.0;
  const double g = 1.0 / std::sqrt(3.0);
  const double pts[2] = {-g, +g};
  const double half = h / 2.0, detJ = half * half * half, s = 2.0 / h;
  std::memset(ke, 0, sizeof(double) * 576);
  for (int ig = 0; ig < 2; ++ig)
    for (int jg = 0; jg < 2; ++jg)
      for (int kg = 0; kg < 2; ++kg) {
        const double xi = pts[ig], eta = pts[jg], zeta = pts[kg];
        double dx[8], dy[8], dz[8];
        for (int a = 0; a < 8; ++a) {
          dx[a] = s * (0.125 * kXi[a] * (1.0 + eta * kEta[a]) * (1.0 + zeta * kZeta[a]));
          dy[a] = s * (0.125 * kEta[a] * (1.0 + xi * kXi[a]) * (1.0 + zeta * kZeta[a]));
          dz[a] = s * (0.125 * kZeta[a] * (1.0 + xi * kXi[a]) * (1.0 + eta * kEta[a]));
        }
        double B[6][24] = {};
        for (int a = 0; a < 8; ++a) {
          B[0][3 * a] = dx[a];
          B[1][3 * a + 1] = dy[a];
          B[2][3 * a + 2] = dz[a];
          B[3][3 * a] = dy[a];
          B[3][3 * a + 1] = dx[a];
          B[4][3 * a + 1] = dz[a];
          B[4][3 * a + 2] = dy[a];
          B[5][3 * a] = dz[a];
          B[5][3 * a + 2] = dx[a];
        }
        double DB[6][24];
        for (int r = 0; r < 6; ++r)
          for (int col = 0; col < 24; ++col) {
            double acc = 0.0;
            for (int m = 0; m < 6; ++m) acc += D[r][m] * B[m][col];
            DB[r][col] = acc;
          }
        for (int r = 0; r < 24; ++r)
          for (int col = 0; col < 24; ++col) {
            double acc = 0.0;
            for (int m = 0; m < 6; ++m) acc += B[m][r] * DB[m][col];
            ke[r * 24 + col] += acc * detJ;
          }
      }
}

// ------------------------------------------------------------- FineProblem
// fn(lo, hi) over [0, n) split across host threads (serial below 64K items).
// The loops it runs are integer and boolean work with per-thread results
// combined exactly, so the outcome does not depend on the split.
template <class F>
static void host_parallel(int64_t n, F&& fn) {
  const unsigned hc = std::thread::hardware_concurrency();
  const int nt = int(std::max(1u, std::min(16u, hc)));
  if (n < (int64_t(1) << 16) || nt == 1) {
    fn(0, n, 0);
    return;
  }
  std::vector<std::thread> th;
  th.reserve(size_t(nt));
  const int64_t chunk = (n + nt - 1) / nt;
  int t = 0;
  for (; t < nt; ++t) {
    const int64_t lo = t * chunk, hi = std::min(n, lo + chunk);
    if (lo >= hi) continue;
    try {
      th.emplace_back([&fn, lo, hi, t] { fn(lo, hi, t); });
    } catch (const std::system_error&) {
      break;  // no thread to be had (many jobs building at once): the rest runs here
    }
  }
  for (; t < nt; ++t) {
    const int64_t lo = t * chunk, hi = std::min(n, lo + chunk);
    if (lo < hi) fn(lo, hi, t);
  }
  for (std::thread& x : th) x.join();
}

void FineProblem::build(const tg_grid& grid, double poisson, const tg_dirichlet_bc* bcs, int nbc,
                        const tg_nodal_load* loads, int nloads, const uint8_t* active_mask,
                        cudaStream_t s) {
  if (grid.nx < 1 || grid.ny < 1 || grid.nz < 1) raise(TG_EINVAL, "grid dimensions must be >= 1");
  if (!(grid.spacing > 0.0)) raise(TG_EINVAL, "hex8_stiffness: element_size must be > 0");
  if (!(poisson > -1.0 && poisson < 0.5))
    raise(TG_EINVAL, "hex8_stiffness: poisson must be in (-1, 0.5)");
  if (nbc < 0 || nloads < 0 || (nbc > 0 && !bcs) || (nloads > 0 && !loads))
    raise(TG_EINVAL, "bcs/loads arrays do not match their counts");
  g = Grid::make(grid.nx, grid.ny, grid.nz, grid.spacing);
  nu = poisson;
  mc = ModalConsts::make(nu, g.h);
  ke.assign(576, 0.0);
  hex8_ke(1.0, nu, g.h, ke.data());
  mc.kdiag = ke[0];
  elem_h.resize(size_t(g.nv));
  host_parallel(g.nv, [&](int64_t lo, int64_t hi, int) {
    for (int64_t e = lo; e < hi; ++e)
      elem_h[size_t(e)] = uint8_t((grid.tags == nullptr || grid.tags[e] != 0) &&
                                  (active_mask == nullptr || active_mask[e] != 0));
  });
  std::vector<uint8_t>& fixed = fixed_h;
  fixed.assign(size_t(g.ndof), 0);
  std::vector<uint8_t> touched(size_t(g.nnodes), 0);
  up_h.assign(size_t(g.ndof), 0.0);
  f_h.assign(size_t(g.ndof), 0.0);
  nonzero_bc = false;
  for (int b = 0; b < nbc; ++b) {
    if (bcs[b].node < 0 || bcs[b].node >= g.nnodes || bcs[b].component < 0 || bcs[b].component > 2)
      raise(TG_EINVAL, "BC index out of range");
    const int64_t d = 3 * int64_t(bcs[b].node) + bcs[b].component;
    fixed[size_t(d)] = 1;
    up_h[size_t(d)] = bcs[b].value;
    if (bcs[b].value != 0.0) nonzero_bc = true;
  }
  for (int l = 0; l < nloads; ++l) {
    if (loads[l].node < 0 || loads[l].node >= g.nnodes || loads[l].component < 0 ||
        loads[l].component > 2)
      raise(TG_EINVAL, "load index out of range");
    f_h[size_t(3 * int64_t(loads[l].node) + loads[l].component)] += loads[l].value;
  }
  // A node is touched when one of its (up to 8) elements exists.
  host_parallel(g.nnodes, [&](int64_t lo, int64_t hi, int) {
    for (int64_t n = lo; n < hi; ++n) {
      const int a = int(n % g.nnx), b = int((n / g.nnx) % g.nny), c = int(n / (int64_t(g.nnx) * g.nny));
      uint8_t t = 0;
      for (int q = 0; q < 8 && !t; ++q) {
        const int i = a - (q & 1), j = b - ((q >> 1) & 1), k = c - (q >> 2);
        if (i >= 0 && i < g.nx && j >= 0 && j < g.ny && k >= 0 && k < g.nz)
          t = elem_h[size_t((int64_t(k) * g.ny + j) * g.nx + i)];
      }
      touched[size_t(n)] = t;
    }
  });
  kept_h.resize(size_t(g.ndof));
  struct Part {
    int64_t n_free = 0, n_touched_free = 0;
    double rmax = 0.0;
    bool void_load = false;
  };
  Part part[16];
  host_parallel(g.ndof, [&](int64_t lo, int64_t hi, int t) {
    Part p;
    for (int64_t d = lo; d < hi; ++d) {
      uint8_t k = 0;
      if (!fixed[size_t(d)]) {
        ++p.n_free;
        p.rmax = std::max(p.rmax, std::fabs(f_h[size_t(d)]));
        if (touched[size_t(d / 3)]) {
          ++p.n_touched_free;
          k = 1;
        }
      }
      kept_h[size_t(d)] = k;
    }
    part[t] = p;
  });
  ng = 0;
  n_free = 0;
  int64_t n_touched_free = 0;
  double rmax = 0.0;
  for (const Part& p : part) {
    n_free += p.n_free;
    n_touched_free += p.n_touched_free;
    ng += p.n_touched_free;
    rmax = std::max(rmax, p.rmax);
  }
  if (n_free > 0 && n_touched_free == 0)
    raise(TG_ESINGULAR, "singular system (no stiffness \xe2\x80\x94 every free DOF is void)");
  const double load_tol = 1e-9 * rmax;
  if (!nonzero_bc) {
    host_parallel(g.ndof, [&](int64_t lo, int64_t hi, int t) {
      bool v = false;
      for (int64_t d = lo; d < hi && !v; ++d)
        v = !fixed[size_t(d)] && !touched[size_t(d / 3)] && std::fabs(f_h[size_t(d)]) > load_tol;
      part[t].void_load = v;
    });
    for (const Part& p : part)
      if (p.void_load)
        raise(TG_ESINGULAR,
              "under-constrained system (load applied to a void DOF with no stiffness \xe2\x80\x94 "
              "no equilibrium possible)");
  }
  // The kept mask once more as 3 bits per node (bit k: DOF 3n+k kept) for the
  // FP32 column operator, which reads one byte per node instead of three.
  kept_node_h.resize(size_t(g.nnodes));
  host_parallel(g.nnodes, [&](int64_t lo, int64_t hi, int) {
    for (int64_t n = lo; n < hi; ++n)
      kept_node_h[size_t(n)] = uint8_t(kept_h[size_t(3 * n)] | kept_h[size_t(3 * n + 1)] << 1 |
                                       kept_h[size_t(3 * n + 2)] << 2);
  });
  elem.alloc(size_t(g.nv));
  kept.alloc(size_t(g.ndof));
  kept_node.alloc(size_t(g.nnodes));
  f.alloc(size_t(g.ndof));
  up.alloc(size_t(g.ndof));
  TG_CUDA(cudaMemcpyAsync(elem.p, elem_h.data(), elem.bytes(), cudaMemcpyHostToDevice, s));
  TG_CUDA(cudaMemcpyAsync(kept.p, kept_h.data(), kept.bytes(), cudaMemcpyHostToDevice, s));
  TG_CUDA(cudaMemcpyAsync(kept_node.p, kept_node_h.data(), kept_node.bytes(),
                          cudaMemcpyHostToDevice, s));
  TG_CUDA(cudaMemcpyAsync(f.p, f_h.data(), f.bytes(), cudaMemcpyHostToDevice, s));
  TG_CUDA(cudaMemcpyAsync(up.p, up_h.data(), up.bytes(), cudaMemcpyHostToDevice, s));
  TG_CUDA(cudaStreamSynchronize(s));
}

size_t FineProblem::device_bytes() const {
  return elem.bytes() + kept.bytes() + kept_node.bytes() + f.bytes() + up.bytes();
}

// ------------------------------------------------------------------ levels
struct Solver::Level {
  MgDims d{};
  int64_t nn = 0, ndof = 0, nel = 0, nact = 0;
  std::vector<uint8_t> act_h;
  DBuf<uint8_t> act;
  // FP64 operators and vectors (plain form, and the FP64 retry of the mixed form).
  DBuf<double> Kel, A, invd, xa, xb, b;
  // FP32 operators and vectors (mixed form).
  DBuf<float> Kelf, Af, invdf, fxa, fxb, fb;
  DBuf<float> chd;  // Chebyshev direction (mixed form, levels >= 2)
  double *x = nullptr, *r = nullptr;
  float *xf = nullptr, *rf = nullptr;
  template <class T>
  void ensure();
  template <class T>
  T*& X();
  template <class T>
  T*& R();
  template <class T>
  T* B();
  template <class T>
  T* Am();
  template <class T>
  T* Dinv();
  template <class T>
  T* Ke();
  size_t bytes() const {
    return act.bytes() + Kel.bytes() + A.bytes() + invd.bytes() + xa.bytes() + xb.bytes() +
           b.bytes() + Kelf.bytes() + Af.bytes() + invdf.bytes() + fxa.bytes() + fxb.bytes() +
           chd.bytes() +
           fb.bytes();
  }
};
template <>
void Solver::Level::ensure<double>() {
  if (Kel.p) return;
  Kel.alloc(size_t(nel) * 576);
  A.alloc(size_t(nn) * kStencilEntries);
  for (DBuf<double>* v : {&invd, &xa, &xb, &b}) v->alloc(size_t(ndof));
  x = xa.p;
  r = xb.p;
}
template <>
void Solver::Level::ensure<float>() {
  if (Kelf.p) return;
  Kelf.alloc(size_t(nel) * 576);
  Af.alloc(size_t(nn) * kStencilEntries);
  for (DBuf<float>* v : {&invdf, &fxa, &fxb, &fb}) v->alloc(size_t(ndof));
  xf = fxa.p;
  rf = fxb.p;
}
template <>
double*& Solver::Level::X<double>() { return x; }
template <>
float*& Solver::Level::X<float>() { return xf; }
template <>
double*& Solver::Level::R<double>() { return r; }
template <>
float*& Solver::Level::R<float>() { return rf; }
template <>
double* Solver::Level::B<double>() { return b.p; }
template <>
float* Solver::Level::B<float>() { return fb.p; }
template <>
double* Solver::Level::Am<double>() { return A.p; }
template <>
float* Solver::Level::Am<float>() { return Af.p; }
template <>
double* Solver::Level::Dinv<double>() { return invd.p; }
template <>
float* Solver::Level::Dinv<float>() { return invdf.p; }
template <>
double* Solver::Level::Ke<double>() { return Kel.p; }
template <>
float* Solver::Level::Ke<float>() { return Kelf.p; }

// ------------------------------------------------------------------ Solver
Solver::Solver(const FineProblem& fp, const tg_solve_options& opt, cudaStream_t s)
    : fp_(fp), opt_(opt), s_(s) {
  omega_ = opt.omega > 0.0 ? opt.omega : 0.6;
  budget_ = opt.mg_iter_budget > 0 ? opt.mg_iter_budget : 300;
  sweeps_ = opt.smooth_sweeps > 0 ? opt.smooth_sweeps : 1;
  df_residual_ = opt.mixed_residual != TG_RESIDUAL_FP64;
  mixed_ = opt.precision == TG_PREC_MIXED;
  // Coarse levels >= 2 of the FP32 V-cycle: Chebyshev by default on grids of
  // >= 200K elements (below that the extra launches of the small levels cost
  // more than the PCG iterations they save), damped Jacobi otherwise.
  const bool cheb = opt.coarse_smoother == TG_SMOOTHER_CHEBYSHEV ||
                    (opt.coarse_smoother == TG_SMOOTHER_AUTO && fp.g.nv >= 200000);
  cheb_m_ = (mixed_ && cheb) ? 4 : 0;
  const size_t n = size_t(fp.g.ndof);
  for (DBuf<double>* b : {&invdiag_, &rhs_, &x_, &r_, &z_, &p_, &ap_, &t0_, &t1_}) b->alloc(n);
  part_n_ = std::max({kRedBlocks, fine_op_blocks(fp.g, true), fine_op_blocks(fp.g, false),
                      152 * 32});
  part_.alloc(size_t(part_n_));
  scal_.alloc(32);
  h_scal_ = static_cast<double*>(pinned_scalars(32 * sizeof(double)));
  istate_.alloc(4);
  h_ist_ = static_cast<int*>(pinned_scalars(4 * sizeof(int)));
  use_graph_ = opt.graph_mode != TG_GRAPH_OFF;
  if (mixed_) {
    Ef_.alloc(size_t(fp.g.nv));
    for (DBuf<float>* b : {&invdiagf_, &xf_, &rf_, &zf_, &pf_, &apf_, &t0f_, &t1f_}) b->alloc(n);
    // Large grids: the FP32 operator's tile shape and z-chunk are measured on
    // first use of the grid's dimensions in the process (a few ms; smaller
    // grids keep the default schedule).
    if (fp.g.nv >= kAutotuneMinVoxels && !fine_schedule_known(fp.g)) {
      launch_fill<float>(Ef_.p, 1.0f, fp.g.nv, s_);
      launch_fill<float>(pf_.p, 1.0f, fp.g.ndof, s_);
      launch_fill<float>(t0f_.p, 0.5f, fp.g.ndof, s_);
      launch_fill<float>(t1f_.p, 0.25f, fp.g.ndof, s_);
      autotune_fine_schedule(fp.g, fp.mc, Ef_.p, fp.kept.p, fp.kept_node.p, pf_.p, apf_.p,
                             part_.p, s_, t0f_.p, t1f_.p);
    }
  }
  if (opt.solver == TG_SOLVER_MGCG) build_structure();
}

struct Solver::InnerGraph {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int64_t body_launches = 0;  // kernels per body execution
  ~InnerGraph() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
  }
};

Solver::~Solver() {
  ig_.reset();
  for (size_t i = 0; i < pi_streams_.size(); ++i) {
    cudaStreamSynchronize(pi_streams_[i]);
    cudaStreamDestroy(pi_streams_[i]);
    cudaEventDestroy(pi_events_[i]);
  }
  if (pi_fork_) cudaEventDestroy(pi_fork_);
  if (s2_) {
    cudaStreamSynchronize(s2_);
    cudaEventDestroy(ev_fork_);
    cudaEventDestroy(ev_join_);
    cudaStreamDestroy(s2_);
  }
  pinned_release(h_scal_);
  pinned_release(h_ist_);
}

size_t Solver::device_bytes() const {
  size_t b = 0;
  for (const DBuf<double>* d : {&invdiag_, &rhs_, &x_, &r_, &z_, &p_, &ap_, &t0_, &t1_, &part_,
                                &scal_, &keb_, &G_, &chol_, &chol_work_})
    b += d->bytes();
  b += chol_li_.bytes() + chol_inv_.bytes() + cdof_.bytes();
  for (const DBuf<float>* d : {&Ef_, &invdiagf_, &xf_, &rf_, &zf_, &pf_, &apf_, &t0f_, &t1f_})
    b += d->bytes();
  for (const auto& L : levels_) b += L->bytes();
  b += spos1_.bytes() + slist1_.bytes() + yspec1_.bytes() + tc_err_.bytes() + chc_.bytes() +
       pipart_.bytes();
  return b + cidx_.bytes() + kebf_.bytes() + Gf_.bytes();
}

void Solver::build_structure() {
  const Grid& g = fp_.g;
  const int max_levels = opt_.mg_levels > 0 ? opt_.mg_levels : 64;
  // Odd axes: the reference's padding (the plain form's default) or the
  // boundary-aligned coarse grid (the mixed form's default); see MgDims::align.
  const int align = opt_.coarsening == TG_COARSEN_ALIGNED ||
                    (opt_.coarsening == TG_COARSEN_DEFAULT && mixed_);
  std::vector<MgDims> dims{dims_of(g.nx, g.ny, g.nz)};
  // Halve (rounding up) while every coarse axis keeps >= 2 elements
  // (kMgMinCoarseElems, coarsen.hpp:80); a requested depth below what keeps the
  // coarsest level dense-factorable is deepened.
  while (true) {
    const MgDims& d = dims.back();
    const int cx = (d.ex + 1) / 2, cy = (d.ey + 1) / 2, cz = (d.ez + 1) / 2;
    if (cx < 2 || cy < 2 || cz < 2) break;
    const int64_t dof_here = 3 * int64_t(d.nnx) * d.nny * d.nnz;
    if (int(dims.size()) >= max_levels && dof_here <= kMaxCoarseDof) break;
    dims.push_back(dims_of(cx, cy, cz));
    dims.back().align = align;
  }
  if (dims.size() < 2) return;
  std::vector<uint8_t> prev = fp_.kept_h;
  MgDims pd = dims[0];
  for (size_t l = 1; l < dims.size(); ++l) {
    auto L = std::make_unique<Level>();
    L->d = dims[l];
    L->nn = int64_t(L->d.nnx) * L->d.nny * L->d.nnz;
    L->ndof = 3 * L->nn;
    L->nel = int64_t(L->d.ex) * L->d.ey * L->d.ez;
    L->act_h.assign(size_t(L->ndof), 0);
    for (int c = 0; c < L->d.nnz; ++c)
      for (int b = 0; b < L->d.nny; ++b)
        for (int a = 0; a < L->d.nnx; ++a) {
          // Coincident fine node; on an aligned odd axis the last coarse node
          // sits on the last fine node.
          auto co = [&](int i, int ef) { return (align && (ef & 1) && i == (ef + 1) / 2) ? ef : 2 * i; };
          const int fa = co(a, pd.ex), fb = co(b, pd.ey), fc = co(c, pd.ez);
          if (fa >= pd.nnx || fb >= pd.nny || fc >= pd.nnz) continue;  // pad node
          const int64_t fn = (int64_t(fc) * pd.nny + fb) * pd.nnx + fa;
          const int64_t cn = (int64_t(c) * L->d.nny + b) * L->d.nnx + a;
          for (int k = 0; k < 3; ++k)
            if (prev[size_t(3 * fn + k)]) {
              L->act_h[size_t(3 * cn + k)] = 1;
              ++L->nact;
            }
        }
    if (L->nact == 0) break;  // multigrid.cpp:1404: nothing left to coarsen onto
    prev = L->act_h;
    pd = L->d;
    levels_.push_back(std::move(L));
  }
  if (levels_.empty()) return;
  // Coarsest compact numbering; too large for a dense factor -> no hierarchy.
  Level& C = *levels_.back();
  std::vector<int> cidx(size_t(C.ndof), -1);
  nc_ = 0;
  for (int64_t d = 0; d < C.ndof; ++d)
    if (C.act_h[size_t(d)]) cidx[size_t(d)] = nc_++;
  if (nc_ > kMaxCoarseDof || nc_ == 0) {
    levels_.clear();
    return;
  }
  for (auto& Lp : levels_) {
    Level& L = *Lp;
    L.act.alloc(size_t(L.ndof));
    TG_CUDA(cudaMemcpyAsync(L.act.p, L.act_h.data(), L.act.bytes(), cudaMemcpyHostToDevice, s_));
    if (mixed_)
      L.ensure<float>();
    else
      L.ensure<double>();
  }
  cidx_.alloc(size_t(C.ndof));
  TG_CUDA(cudaMemcpyAsync(cidx_.p, cidx.data(), cidx_.bytes(), cudaMemcpyHostToDevice, s_));
  std::vector<int> cdof(static_cast<size_t>(nc_));
  for (int64_t d = 0; d < C.ndof; ++d)
    if (cidx[size_t(d)] >= 0) cdof[size_t(cidx[size_t(d)])] = int(d);
  cdof_.alloc(size_t(nc_));
  TG_CUDA(cudaMemcpyAsync(cdof_.p, cdof.data(), cdof_.bytes(), cudaMemcpyHostToDevice, s_));
  if (nc_ <= kMaxInverseDof) {
    chol_li_.alloc(size_t(nc_) * nc_);
    chol_inv_.alloc(size_t(nc_) * nc_);
  }
  chol_.alloc(size_t(nc_) * nc_);
  chol_work_.alloc(size_t(nc_));
  chol_fail_.alloc(1);
  // Ke in corner-bit order and the 8 child Galerkin blocks G_c = W_c^T Ke W_c.
  std::vector<double> kb(576);
  for (int a = 0; a < 8; ++a)
    for (int b = 0; b < 8; ++b)
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
          kb[size_t((3 * kLocToBit[a] + i) * 24 + 3 * kLocToBit[b] + j)] =
              fp_.ke[size_t((3 * a + i) * 24 + 3 * b + j)];
  auto w1 = [](int pos, int t) { return pos == 1 ? 0.5 : ((pos == 0) == (t == 0) ? 1.0 : 0.0); };
  std::vector<double> G(8 * 576, 0.0);
  for (int ch = 0; ch < 8; ++ch) {
    double W[8][8];
    for (int sc = 0; sc < 8; ++sc)
      for (int t = 0; t < 8; ++t)
        W[sc][t] = w1((ch & 1) + (sc & 1), t & 1) * w1(((ch >> 1) & 1) + ((sc >> 1) & 1), (t >> 1) & 1) *
                   w1((ch >> 2) + (sc >> 2), t >> 2);
    for (int t1 = 0; t1 < 8; ++t1)
      for (int c1 = 0; c1 < 3; ++c1)
        for (int t2 = 0; t2 < 8; ++t2)
          for (int c2 = 0; c2 < 3; ++c2) {
            double acc = 0.0;
            for (int s1 = 0; s1 < 8; ++s1) {
              if (W[s1][t1] == 0.0) continue;
              for (int s2 = 0; s2 < 8; ++s2)
                acc += W[s1][t1] * W[s2][t2] * kb[size_t((3 * s1 + c1) * 24 + 3 * s2 + c2)];
            }
            G[size_t(ch * 576 + (3 * t1 + c1) * 24 + 3 * t2 + c2)] = acc;
          }
  }
  keb_.alloc(576);
  G_.alloc(8 * 576);
  TG_CUDA(cudaMemcpyAsync(keb_.p, kb.data(), keb_.bytes(), cudaMemcpyHostToDevice, s_));
  TG_CUDA(cudaMemcpyAsync(G_.p, G.data(), G_.bytes(), cudaMemcpyHostToDevice, s_));
  std::vector<float> kbf(kb.begin(), kb.end()), Gf(G.begin(), G.end());
  kebf_.alloc(576);
  Gf_.alloc(8 * 576);
  TG_CUDA(cudaMemcpyAsync(kebf_.p, kbf.data(), kebf_.bytes(), cudaMemcpyHostToDevice, s_));
  TG_CUDA(cudaMemcpyAsync(Gf_.p, Gf.data(), Gf_.bytes(), cudaMemcpyHostToDevice, s_));
  l1_tc_ = mixed_ && level1_tc_enabled();
  if (l1_tc_) {
    // Coarse elements of level 1 off the sum_c E_c G_c fast path.
    const Level& L1 = *levels_[0];
    const MgDims& d = L1.d;
    std::vector<uint8_t> spec(size_t(L1.nel), 0);
    host_parallel(L1.nel, [&](int64_t lo, int64_t hi, int) {
      for (int64_t ce = lo; ce < hi; ++ce) {
        const int I = int(ce % d.ex), J = int((ce / d.ex) % d.ey), K = int(ce / (int64_t(d.ex) * d.ey));
        bool sp = d.align && ((2 * I + 1 == g.nx) || (2 * J + 1 == g.ny) || (2 * K + 1 == g.nz));
        for (int c = 0; c < 8 && !sp; ++c) {
          const int64_t cn = (int64_t(K + (c >> 2)) * d.nny + (J + ((c >> 1) & 1))) * d.nnx +
                             (I + (c & 1));
          for (int k = 0; k < 3; ++k)
            if (!L1.act_h[size_t(3 * cn + k)]) sp = true;
        }
        for (int ch = 0; ch < 8 && !sp; ++ch) {
          const int fi = 2 * I + (ch & 1), fj = 2 * J + ((ch >> 1) & 1), fk = 2 * K + (ch >> 2);
          if (fi >= g.nx || fj >= g.ny || fk >= g.nz) continue;
          if (!fp_.elem_h[size_t((int64_t(fk) * g.ny + fj) * g.nx + fi)]) continue;
          for (int c = 0; c < 8 && !sp; ++c) {
            const int64_t fn = (int64_t(fk + (c >> 2)) * g.nny + (fj + ((c >> 1) & 1))) * g.nnx +
                               (fi + (c & 1));
            for (int k = 0; k < 3; ++k)
              if (!fp_.kept_h[size_t(3 * fn + k)]) sp = true;
          }
        }
        spec[size_t(ce)] = uint8_t(sp);
      }
    });
    std::vector<int> spos(spec.size(), -1), slist;
    for (size_t ce = 0; ce < spec.size(); ++ce)
      if (spec[ce]) {
        spos[ce] = int(slist.size());
        slist.push_back(int(ce));
      }
    nspec1_ = int(slist.size());
    spos1_.alloc(spos.size());
    TG_CUDA(cudaMemcpyAsync(spos1_.p, spos.data(), spos1_.bytes(), cudaMemcpyHostToDevice, s_));
    if (nspec1_ > 0) {
      slist1_.alloc(slist.size());
      yspec1_.alloc(slist.size() * 24);
      TG_CUDA(cudaMemcpyAsync(slist1_.p, slist.data(), slist1_.bytes(), cudaMemcpyHostToDevice,
                              s_));
    }
    tc_err_.alloc(1);
    TG_CUDA(cudaMemsetAsync(tc_err_.p, 0, sizeof(int), s_));
  }
  // The small levels (from the first one of at most kFusedMaxNodes nodes, below
  // level 1) in one cluster launch, when at least one of them is smoothed and
  // the coarsest has the explicit inverse.
  side_level_ = levels_.size() >= 2 ? 2 : 0;
  if (mixed_ && side_level_ > 0) ensure_side();
  fused_level_ = 0;
  if (mixed_ && coarse_fused_enabled() && chol_inv_.p != nullptr) {
    for (size_t l = 2; l < levels_.size(); ++l) {
      const MgDims& d = levels_[l - 1]->d;
      if (int64_t(d.nnx) * d.nny * d.nnz <= kFusedMaxNodes) {
        if (levels_.size() - (l - 1) <= size_t(kFusedMaxLevels)) fused_level_ = l;
        break;
      }
    }
  }
  TG_CUDA(cudaStreamSynchronize(s_));
  have_mg_ = true;
}

// Level 1 of the FP32 V-cycle on the tensor cores (mode kResidual or kSmooth):
// L.R = b - A1 x or the smoothed iterate, as the stencil apply would write it.
void Solver::level1_op(int mode, Level& L, float omega) {
  const Grid& g = fp_.g;
  mg_level1_tc(mode, dims_of(g.nx, g.ny, g.nz), L.d, Ef_.p, L.act.p, spos1_.p, slist1_.p,
               nspec1_, L.Ke<float>(), Gf_.p, L.X<float>(), L.B<float>(), L.Dinv<float>(), omega,
               L.R<float>(), yspec1_.p, tc_err_.p, s_);
}

double Solver::read_scalar(int idx) {
  TG_CUDA(cudaMemcpyAsync(h_scal_ + idx, scal_.p + idx, sizeof(double), cudaMemcpyDeviceToHost, s_));
  TG_CUDA(cudaStreamSynchronize(s_));
  return h_scal_[idx];
}

void Solver::read_scalars(int idx0, int n, double* out) {
  TG_CUDA(cudaMemcpyAsync(h_scal_ + idx0, scal_.p + idx0, sizeof(double) * n,
                          cudaMemcpyDeviceToHost, s_));
  TG_CUDA(cudaStreamSynchronize(s_));
  for (int i = 0; i < n; ++i) out[i] = h_scal_[idx0 + i];
}

void Solver::apply_unmasked(const double* E, const double* x, double* y) {
  launch_fine_op<double>(kApply, fp_.g, fp_.mc, E, nullptr, x, nullptr, nullptr, 0.0, y, nullptr,
                         nullptr, s_);
}

// The assembled FP32 level-1 stencil, formed from the level's element matrices
// if the last hierarchy build kept only its diagonal.
void Solver::level1_stencil() {
  if (l1_stencil_ok_) return;
  Level& L = *levels_[0];
  mg_assemble_stencil<float>(L.d, L.Ke<float>(), L.act.p, L.Am<float>(), L.Dinv<float>(), s_);
  l1_stencil_ok_ = true;
}

double Solver::check_level1() {
  if (!mixed_ || !l1_tc_ || !have_mg_ || !numeric_ok_)
    raise(TG_EINVAL, "check_level1: needs a mixed job with the level-1 tensor-core path");
  level1_stencil();
  Level& L = *levels_[0];
  const size_t n = size_t(L.ndof);
  std::vector<float> xh(n), a(n), bq(n);
  uint64_t h = 0x9E3779B97F4A7C15ull;
  for (size_t i = 0; i < n; ++i) {
    h ^= h << 13;
    h ^= h >> 7;
    h ^= h << 17;
    xh[i] = L.act_h[i] ? float(double(h >> 11) * (1.0 / 9007199254740992.0) - 0.5) : 0.0f;
  }
  TG_CUDA(cudaMemcpyAsync(L.X<float>(), xh.data(), n * sizeof(float), cudaMemcpyHostToDevice, s_));
  mg_stencil_op<float>(kApply, L.d, L.Am<float>(), L.act.p, L.X<float>(), L.B<float>(),
                       L.Dinv<float>(), 0.0f, L.R<float>(), s_);
  TG_CUDA(cudaMemcpyAsync(a.data(), L.R<float>(), n * sizeof(float), cudaMemcpyDeviceToHost, s_));
  TG_CUDA(cudaStreamSynchronize(s_));
  level1_op(kApply, L, 0.0f);
  TG_CUDA(cudaMemcpyAsync(bq.data(), L.R<float>(), n * sizeof(float), cudaMemcpyDeviceToHost, s_));
  int tc_err = 0;
  TG_CUDA(cudaMemcpyAsync(&tc_err, tc_err_.p, sizeof(int), cudaMemcpyDeviceToHost, s_));
  TG_CUDA(cudaStreamSynchronize(s_));
  if (tc_err) raise(TG_EDEVICE, "level-1 tensor-core operator: MMA completion wait timed out");
  double dmax = 0.0, amax = 0.0;
  for (size_t i = 0; i < n; ++i) {
    dmax = std::max(dmax, std::fabs(double(a[i]) - double(bq[i])));
    amax = std::max(amax, std::fabs(double(a[i])));
  }
  return amax > 0.0 ? dmax / amax : dmax;
}

double Solver::time_operator(int form, int reps) {
  const Grid& g = fp_.g;
  const bool fp32 = form == 1;
  if ((fp32 || form >= 3) && !mixed_)
    raise(TG_EINVAL, "time_operator: FP32 operators need a mixed-precision job");
  if (form >= 3) {
    // Level 1 of the FP32 V-cycle, residual mode: form 3 the assembled stencil,
    // form 4 the tensor-core operator.
    if (!have_mg_ || !numeric_ok_) raise(TG_EINVAL, "time_operator: no multigrid hierarchy");
    if (form == 4 && !l1_tc_) raise(TG_EINVAL, "time_operator: level-1 tensor-core path is off");
    if (form == 3) level1_stencil();
    Level& L = *levels_[0];
    launch_fill<float>(L.X<float>(), 1.0f, L.ndof, s_);
    launch_fill<float>(L.B<float>(), 0.5f, L.ndof, s_);
    cudaEvent_t a, b;
    TG_CUDA(cudaEventCreate(&a));
    TG_CUDA(cudaEventCreate(&b));
    TG_CUDA(cudaEventRecord(a, s_));
    for (int i = 0; i < reps; ++i) {
      if (form == 4)
        level1_op(kResidual, L, float(omega_));
      else
        mg_stencil_op<float>(kResidual, L.d, L.Am<float>(), L.act.p, L.X<float>(), L.B<float>(),
                             L.Dinv<float>(), float(omega_), L.R<float>(), s_);
    }
    TG_CUDA(cudaEventRecord(b, s_));
    TG_CUDA(cudaEventSynchronize(b));
    float ms = 0.0f;
    TG_CUDA(cudaEventElapsedTime(&ms, a, b));
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return double(ms) / reps;
  }
  launch_fill<double>(p_.p, 1.0, g.ndof, s_);
  if (fp32) launch_copy_d2f(pf_.p, p_.p, g.ndof, s_);
  cudaEvent_t a, b;
  TG_CUDA(cudaEventCreate(&a));
  TG_CUDA(cudaEventCreate(&b));
  TG_CUDA(cudaEventRecord(a, s_));
  for (int i = 0; i < reps; ++i) {
    if (fp32)
      launch_fine_op<float>(kApply, g, fp_.mc, Ef_.p, fp_.kept.p, pf_.p, nullptr, nullptr, 0.0f,
                            apf_.p, nullptr, nullptr, s_, fp_.kept_node.p);
    else if (form == 2)  // the double-float residual kernel
      launch_fine_residual_df(g, fp_.mc, E_, fp_.kept.p, p_.p, rhs_.p, ap_.p, s_);
    else
      launch_fine_op<double>(kApply, g, fp_.mc, E_, fp_.kept.p, p_.p, nullptr, nullptr, 0.0,
                             ap_.p, nullptr, nullptr, s_);
  }
  TG_CUDA(cudaEventRecord(b, s_));
  TG_CUDA(cudaEventSynchronize(b));
  float ms = 0.0f;
  TG_CUDA(cudaEventElapsedTime(&ms, a, b));
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return double(ms) / reps;
}

void Solver::set_modulus(const double* E) {
  E_ = E;
  const Grid& g = fp_.g;
  launch_fine_invdiag(g, fp_.mc.kdiag, E, fp_.kept.p, invdiag_.p, s_);
  // rhs = f - K u_p on the kept DOFs (matfree.cpp:740-750).
  if (fp_.nonzero_bc) {
    apply_unmasked(E, fp_.up.p, t0_.p);
  } else {
    launch_fill<double>(t0_.p, 0.0, g.ndof, s_);
  }
  launch_sub_mask(rhs_.p, fp_.f.p, t0_.p, fp_.kept.p, g.ndof, s_);
  if (fp_.nonzero_bc) {
    // The void-load check on the full right-hand side f - K u_p, rmax over the
    // free DOFs (matfree.cpp:796-814).
    std::vector<double> kup(size_t(g.ndof));
    TG_CUDA(cudaMemcpyAsync(kup.data(), t0_.p, t0_.bytes(), cudaMemcpyDeviceToHost, s_));
    TG_CUDA(cudaStreamSynchronize(s_));
    double rmax = 0.0;
    for (int64_t d = 0; d < g.ndof; ++d)
      if (!fp_.fixed_h[size_t(d)])
        rmax = std::max(rmax, std::fabs(fp_.f_h[size_t(d)] - kup[size_t(d)]));
    for (int64_t d = 0; d < g.ndof; ++d)
      if (!fp_.fixed_h[size_t(d)] && !fp_.kept_h[size_t(d)] &&
          std::fabs(fp_.f_h[size_t(d)] - kup[size_t(d)]) > 1e-9 * rmax)
        raise(TG_ESINGULAR,
              "under-constrained system (load applied to a void DOF with no stiffness \xe2\x80\x94 "
              "no equilibrium possible)");
  }
  if (mixed_) {
    launch_copy_d2f(Ef_.p, E, g.nv, s_);
    launch_copy_d2f(invdiagf_.p, invdiag_.p, g.ndof, s_);
  }
  numeric_[0] = numeric_[1] = false;
  numeric_ok_ = false;
  if (have_mg_) {
    const double t0 = now_ms();
    numeric_ok_ = mixed_ ? build_numeric<float>() : build_numeric<double>();
    mg_build_ms_ = now_ms() - t0;
  }
}

template <class T>
static const T* pick(const DBuf<double>& d, const DBuf<float>& f);
template <>
const double* pick<double>(const DBuf<double>& d, const DBuf<float>&) {
  return d.p;
}
template <>
const float* pick<float>(const DBuf<double>&, const DBuf<float>& f) {
  return f.p;
}

// Galerkin hierarchy in precision T from the current element factors, then the
// FP64 dense Cholesky factor of the coarsest level.  Returns false when the
// factorisation meets a non-positive pivot (the caller falls back).
template <class T>
bool Solver::build_numeric() {
  const Grid& g = fp_.g;
  const MgDims fd = dims_of(g.nx, g.ny, g.nz);
  MgDims pd = fd;
  const T* ef = sizeof(T) == 8 ? reinterpret_cast<const T*>(E_) : reinterpret_cast<const T*>(Ef_.p);
  for (size_t l = 0; l < levels_.size(); ++l) {
    Level& L = *levels_[l];
    L.ensure<T>();
    if (l == 0)
      mg_galerkin_level1<T>(fd, L.d, ef, fp_.kept.p, L.act.p, pick<T>(keb_, kebf_),
                            pick<T>(G_, Gf_), L.Ke<T>(), s_,
                            sizeof(T) == 4 && l1_tc_ && level1_galerkin_fast_enabled()
                                ? spos1_.p
                                : nullptr);
    else
      mg_galerkin_coarse<T>(pd, L.d, levels_[l - 1]->Ke<T>(), L.act.p, L.Ke<T>(), s_);
    // Level 1 on the tensor cores needs only its inverse diagonal; the assembled
    // stencil (275 MB on the 256x128x128 cantilever) is formed on demand (level1_stencil()).
    const bool diag_only = sizeof(T) == 4 && l == 0 && l1_tc_;
    mg_assemble_stencil<T>(L.d, L.Ke<T>(), L.act.p, diag_only ? nullptr : L.Am<T>(), L.Dinv<T>(),
                           s_);
    if (sizeof(T) == 4 && l == 0) l1_stencil_ok_ = !diag_only;
    pd = L.d;
  }
  if (sizeof(T) == 4 && cheb_m_ > 0) {
    // lambda_max(D^-1 A) of every smoothed level >= 2 for its Chebyshev smoother.
    // The levels' power iterations are independent chains of small launches
    // (10 steps of 5 each); they run side by side, one stream per level, each
    // with its own partials, and rejoin the solver's stream.
    const size_t nlev = levels_.size();
    if (!lam_.p) lam_.alloc(nlev + 1);
    if (!chc_.p) chc_.alloc(kChebCoefStride * (nlev + 1));
    constexpr size_t kPiStride = size_t(kRedBlocks) + 8;  // partials, then the norm
    if (!pipart_.p) pipart_.alloc((nlev + 1) * kPiStride);
    ensure_pi_streams(nlev);
    TG_CUDA(cudaEventRecord(pi_fork_, s_));
    for (size_t li = 1; li + 1 < nlev; ++li) {
      Level& L = *levels_[li];
      if (!L.chd.p) L.chd.alloc(size_t(L.ndof));
      cudaStream_t ls = pi_streams_[li];
      double* part = pipart_.p + li * kPiStride;
      TG_CUDA(cudaStreamWaitEvent(ls, pi_fork_, 0));
      mg_lambda_max<float>(L.d, L.Am<float>(), L.act.p, L.Dinv<float>(), L.X<float>(),
                           L.R<float>(), cheb_iters_, cheb_safety_, part, part + kRedBlocks,
                           lam_.p + li, ls);
      mg_cheb_table(lam_.p + li, cheb_ratio_, cheb_m_, chc_.p + kChebCoefStride * li, ls);
      TG_CUDA(cudaEventRecord(pi_events_[li], ls));
      TG_CUDA(cudaStreamWaitEvent(s_, pi_events_[li], 0));
    }
  }
  Level& C = *levels_.back();
  mg_dense_from_stencil<T>(C.d, C.Am<T>(), cidx_.p, nc_, chol_.p, s_);
  TG_CUDA(cudaMemsetAsync(chol_fail_.p, 0, sizeof(int), s_));
  mg_cholesky(chol_.p, nc_, chol_fail_.p, s_);
  int fail = 0;
  TG_CUDA(cudaMemcpyAsync(&fail, chol_fail_.p, sizeof(int), cudaMemcpyDeviceToHost, s_));
  TG_CUDA(cudaStreamSynchronize(s_));
  if (fail == 0 && chol_inv_.p) mg_chol_inverse(chol_.p, nc_, chol_li_.p, chol_inv_.p, s_);
  numeric_[sizeof(T) == 8 ? 1 : 0] = (fail == 0);
  return fail == 0;
}

// ------------------------------------------------------------------ V-cycle
template <class T>
FirstStep<T> Solver::first_step(size_t l) {
  FirstStep<T> f;
  if (l >= levels_.size()) return f;  // the coarsest: solved, not smoothed
  if constexpr (sizeof(T) == 4) {
    if (l == fused_level_) return f;  // the fused launch takes its own first step
  }
  Level& L = *levels_[l - 1];
  f.dinv = L.Dinv<T>();
  if (sizeof(T) == 4 && cheb_m_ > 0 && l >= 2) {
    f.kind = 2;
    f.coef = chc_.p + kChebCoefStride * (l - 1);
    f.x = L.R<T>();  // step 0 writes the other buffer, as the stencil step does
    f.chd = static_cast<T*>(static_cast<void*>(L.chd.p));
  } else {
    f.kind = 1;
    f.omega = T(omega_);
    f.x = L.X<T>();
  }
  return f;
}

// One stream and event per level for the power iterations of the hierarchy
// build (never inside a capture), and the event they fork from.
void Solver::ensure_pi_streams(size_t nlev) {
  if (!pi_fork_) TG_CUDA(cudaEventCreateWithFlags(&pi_fork_, cudaEventDisableTiming));
  while (pi_streams_.size() < nlev) {
    cudaStream_t st = nullptr;
    cudaEvent_t ev = nullptr;
    TG_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    TG_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    pi_streams_.push_back(st);
    pi_events_.push_back(ev);
  }
}

// The side stream (lowest priority) and its two events; created before any
// capture begins, never inside one.
void Solver::ensure_side() {
  if (s2_) return;
  int lo = 0, hi = 0;
  TG_CUDA(cudaDeviceGetStreamPriorityRange(&lo, &hi));
  TG_CUDA(cudaStreamCreateWithPriority(&s2_, cudaStreamNonBlocking, lo));
  TG_CUDA(cudaEventCreateWithFlags(&ev_fork_, cudaEventDisableTiming));
  TG_CUDA(cudaEventCreateWithFlags(&ev_join_, cudaEventDisableTiming));
}

bool Solver::fork_x() {
  if (!pending_x_ || !s2_) return false;
  TG_CUDA(cudaEventRecord(ev_fork_, s_));
  TG_CUDA(cudaStreamWaitEvent(s2_, ev_fork_, 0));
  launch_cg_update_x_f(xf_.p, pf_.p, scal_.p + 6, scal_.p + 7, fp_.g.ndof, s2_);
  TG_CUDA(cudaEventRecord(ev_join_, s2_));
  pending_x_ = false;
  side_joined_ = false;
  return true;
}

// Called from a destructor while an error may be propagating: no throw; a
// failed wait leaves the error for the next checked call.
void Solver::join_x() noexcept {
  if (side_joined_) return;
  cudaStreamWaitEvent(s_, ev_join_, 0);
  side_joined_ = true;
}

void Solver::flush_x() {
  if (!pending_x_) return;
  launch_cg_update_x_f(xf_.p, pf_.p, scal_.p + 6, scal_.p + 7, fp_.g.ndof, s_);
  pending_x_ = false;
}

// first_done: the restriction into this level already took its first smoothing
// step from zero (first_step).
template <class T>
T* Solver::vcycle_level(size_t l, bool first_done) {
  Level& L = *levels_[l - 1];
  // The pending x += alpha p of the FP32 PCG runs on the side stream while this
  // level and the ones below it work (latency-bound launches that leave HBM
  // idle); it joins the solver's stream when this level returns.
  struct SideJoin {
    Solver* s;
    bool on;
    ~SideJoin() {
      if (on) s->join_x();
    }
  } side{this, false};
  if constexpr (sizeof(T) == 4) {
    if (l == side_level_ && pending_x_) side.on = fork_x();
  }
  if (l == levels_.size()) {
    if (chol_inv_.p)
      mg_coarse_inv_apply<T>(chol_inv_.p, nc_, cidx_.p, cdof_.p, L.ndof, L.B<T>(), L.X<T>(), s_);
    else
      mg_chol_solve<T>(chol_.p, nc_, cidx_.p, L.ndof, L.B<T>(), L.X<T>(), chol_work_.p, s_);
    return L.X<T>();
  }
  if constexpr (sizeof(T) == 4) {
    if (l == fused_level_) return reinterpret_cast<T*>(fused_coarse_vcycle());
  }
  Level& N = *levels_[l];
  const T w = T(omega_);
  auto op = [&](int mode) {
    if constexpr (sizeof(T) == 4) {
      if (l == 1 && l1_tc_) {
        level1_op(mode, L, float(w));
        return;
      }
    }
    mg_stencil_op<T>(mode, L.d, L.Am<T>(), L.act.p, L.X<T>(), L.B<T>(), L.Dinv<T>(), w, L.R<T>(),
                     s_);
  };
  if (sizeof(T) == 4 && cheb_m_ > 0 && l >= 2) {
    // Mixed form, levels >= 2: a degree-cheb_m_ Chebyshev polynomial in D^-1 A
    // before (from a zero iterate) and after the coarse correction.
    ChebStep ch{L.chd.p, chc_.p + kChebCoefStride * (l - 1), 0};
    auto cheb = [&](int k0) {
      for (int k = k0; k < cheb_m_; ++k) {
        ch.step = k;
        mg_stencil_op<T>(kCheb, L.d, L.Am<T>(), L.act.p, L.X<T>(), L.B<T>(), L.Dinv<T>(), w,
                         L.R<T>(), s_, ch);
        std::swap(L.X<T>(), L.R<T>());
      }
    };
    if (first_done) {
      std::swap(L.X<T>(), L.R<T>());
      cheb(1);
    } else {
      launch_fill<T>(L.X<T>(), T(0), L.ndof, s_);
      cheb(0);
    }
    op(kResidual);
    const FirstStep<T> fs = first_step<T>(l + 1);
    mg_restrict<T>(L.d, N.d, L.R<T>(), N.act.p, N.B<T>(), s_, fs);
    T* ec = vcycle_level<T>(l + 1, fs.kind != 0);
    mg_prolong_add<T>(L.d, N.d, ec, L.act.p, L.X<T>(), s_);
    cheb(0);
    return L.X<T>();
  }
  // sweeps_ damped-Jacobi sweeps on each side (the first from a zero iterate);
  // every sweep leaves the iterate in X.
  if (!first_done) mg_jacobi_first<T>(L.B<T>(), L.Dinv<T>(), w, L.ndof, L.X<T>(), s_);
  for (int k = 1; k < sweeps_; ++k) {
    op(kSmooth);
    std::swap(L.X<T>(), L.R<T>());
  }
  op(kResidual);
  const FirstStep<T> fs = first_step<T>(l + 1);
  mg_restrict<T>(L.d, N.d, L.R<T>(), N.act.p, N.B<T>(), s_, fs);
  T* ec = vcycle_level<T>(l + 1, fs.kind != 0);
  mg_prolong_add<T>(L.d, N.d, ec, L.act.p, L.X<T>(), s_);
  for (int k = 0; k < sweeps_; ++k) {
    op(kSmooth);
    std::swap(L.X<T>(), L.R<T>());
  }
  return L.X<T>();
}

// Levels fused_level_ .. coarsest of the FP32 V-cycle as one cluster launch;
// returns the buffer that holds level fused_level_'s result (the launch-by-launch
// V-cycle leaves it in the same one).
float* Solver::fused_coarse_vcycle() {
  FusedCoarse fc;
  const size_t first = fused_level_ - 1;  // levels_ index of the first fused level
  fc.nlev = int(levels_.size() - first);
  for (int i = 0; i < fc.nlev; ++i) {
    Level& L = *levels_[first + size_t(i)];
    FusedLevel& F = fc.L[i];
    F.d = L.d;
    F.A = L.Am<float>();
    F.act = L.act.p;
    F.dinv = L.Dinv<float>();
    F.xp = L.X<float>();
    F.xq = L.R<float>();
    F.b = L.B<float>();
    F.chd = L.chd.p;
    F.coef = chc_.p ? chc_.p + kChebCoefStride * (first + size_t(i)) : nullptr;
  }
  fc.cheb_m = cheb_m_;
  fc.sweeps = sweeps_;
  fc.omega = float(omega_);
  fc.Ainv = chol_inv_.p;
  fc.nc = nc_;
  fc.cidx = cidx_.p;
  fc.cdof = cdof_.p;
  mg_coarse_vcycle_fused(fc, s_);
  // Chebyshev: 2 cheb_m toggles per level (even); Jacobi: the first sweep in
  // place, then 2 sweeps - 1 toggles (odd).
  return cheb_m_ > 0 ? fc.L[0].xp : fc.L[0].xq;
}

template <>
double* Solver::vcycle<double>(const double* b, double* bz, bool x0_ready) {
  if (bz != nullptr || x0_ready) raise(TG_EINVAL, "vcycle<double>: no fused b.z or first sweep");
  const Grid& g = fp_.g;
  Level& N = *levels_[0];
  const MgDims fd = dims_of(g.nx, g.ny, g.nz);
  double* x = t1_.p;
  double* r = t0_.p;
  auto smooth = [&] {
    launch_fine_op<double>(kSmooth, g, fp_.mc, E_, fp_.kept.p, x, b, invdiag_.p, omega_, r,
                           nullptr, nullptr, s_);
    std::swap(x, r);
  };
  mg_jacobi_first<double>(b, invdiag_.p, omega_, g.ndof, x, s_);
  for (int k = 1; k < sweeps_; ++k) smooth();
  launch_fine_op<double>(kResidual, g, fp_.mc, E_, fp_.kept.p, x, b, invdiag_.p, omega_, r,
                         nullptr, nullptr, s_);
  const FirstStep<double> fs = first_step<double>(1);
  mg_restrict<double>(fd, N.d, r, N.act.p, N.B<double>(), s_, fs);
  double* ec = vcycle_level<double>(1, fs.kind != 0);
  mg_prolong_add<double>(fd, N.d, ec, fp_.kept.p, x, s_);
  for (int k = 0; k < sweeps_; ++k) smooth();
  fine_matvecs_ += 2 * sweeps_;
  return x;
}

template <>
// With bz set, b . z of the returned z is summed into *bz (device): the last
// smoothing sweep accumulates it while it writes z.  With x0_ready the first
// sweep from zero, omega D^-1 b, is already in t1f_ (the PCG's r update wrote
// it).
float* Solver::vcycle<float>(const float* b, double* bz, bool x0_ready) {
  const Grid& g = fp_.g;
  Level& N = *levels_[0];
  const MgDims fd = dims_of(g.nx, g.ny, g.nz);
  float* x = t1f_.p;
  float* r = t0f_.p;
  const float w = float(omega_);
  auto smooth = [&](bool last) {
    int nb = 0;
    double* part = last && bz != nullptr ? part_.p : nullptr;
    launch_fine_op<float>(kSmooth, g, fp_.mc, Ef_.p, fp_.kept.p, x, b, invdiagf_.p, w, r, part,
                          &nb, s_, fp_.kept_node.p);
    if (part != nullptr) launch_sum_partials(part_.p, nb, bz, s_);
    std::swap(x, r);
  };
  if (!x0_ready) mg_jacobi_first<float>(b, invdiagf_.p, w, g.ndof, x, s_);
  for (int k = 1; k < sweeps_; ++k) smooth(false);
  launch_fine_op<float>(kResidual, g, fp_.mc, Ef_.p, fp_.kept.p, x, b, invdiagf_.p, w, r, nullptr,
                        nullptr, s_, fp_.kept_node.p);
  const FirstStep<float> fs = first_step<float>(1);
  mg_restrict<float>(fd, N.d, r, N.act.p, N.B<float>(), s_, fs);
  float* ec = vcycle_level<float>(1, fs.kind != 0);
  mg_prolong_add<float>(fd, N.d, ec, fp_.kept.p, x, s_);
  for (int k = 0; k < sweeps_; ++k) smooth(k == sweeps_ - 1);
  lowp_matvecs_ += 2 * sweeps_;
  return x;
}

// ------------------------------------------------------------------ MG-PCG
// mf_mgpcg (multigrid.cpp:1211-1313): stop at ||r|| <= tol ||b||, breakdown when
// pAp <= 0 or non-finite, x finite at exit.
bool Solver::mgpcg(double tol, int max_it, bool warm, SolverStats& st) {
  const Grid& g = fp_.g;
  const int64_t n = g.ndof;
  launch_dot(rhs_.p, rhs_.p, n, part_.p, scal_.p + 4, s_);
  const double bnorm2 = read_scalar(4);
  st.iterations = 0;
  st.residual = 0.0;
  if (!(bnorm2 > 0.0)) {
    launch_fill<double>(x_.p, 0.0, n, s_);
    return true;
  }
  const double bnorm = std::sqrt(bnorm2), threshold = tol * bnorm;
  if (warm) {
    refinement_residual();
  } else {
    launch_fill<double>(x_.p, 0.0, n, s_);
    TG_CUDA(cudaMemcpyAsync(r_.p, rhs_.p, size_t(n) * sizeof(double), cudaMemcpyDeviceToDevice, s_));
  }
  double* z = vcycle<double>(r_.p);
  TG_CUDA(cudaMemcpyAsync(p_.p, z, size_t(n) * sizeof(double), cudaMemcpyDeviceToDevice, s_));
  launch_dot(r_.p, z, n, part_.p, scal_.p + 0, s_);
  if (!std::isfinite(read_scalar(0))) return false;
  int nb = 0;
  for (int k = 1; k <= max_it; ++k) {
    launch_fine_op<double>(kApply, g, fp_.mc, E_, fp_.kept.p, p_.p, nullptr, nullptr, 0.0, ap_.p,
                           part_.p, &nb, s_);
    ++fine_matvecs_;
    launch_sum_partials(part_.p, nb, scal_.p + 1, s_);
    launch_cg_update_xr<double>(x_.p, r_.p, p_.p, ap_.p, scal_.p + 0, scal_.p + 1, n, part_.p, s_);
    launch_sum_partials(part_.p, kRedBlocks, scal_.p + 2, s_);
    double sc[2];
    read_scalars(1, 2, sc);
    const double pap = sc[0], rr = sc[1];
    if (!(pap > 0.0) || !std::isfinite(pap)) return false;
    st.iterations = k;
    const double rn = std::sqrt(rr);
    st.residual = rn / bnorm;
    if (rn <= threshold) {
      launch_dot(x_.p, x_.p, n, part_.p, scal_.p + 5, s_);
      return std::isfinite(read_scalar(5));
    }
    z = vcycle<double>(r_.p);
    launch_dot(r_.p, z, n, part_.p, scal_.p + 3, s_);
    launch_cg_update_p<double>(p_.p, z, scal_.p + 3, scal_.p + 0, n, s_);
    TG_CUDA(cudaMemcpyAsync(scal_.p + 0, scal_.p + 3, sizeof(double), cudaMemcpyDeviceToDevice, s_));
  }
  return false;
}

// FP32 inner MG-PCG on the unit-norm residual held in zf_; solution in xf_.
// FP64 dot products; stops at relative residual rel_tol or max_it.
// The decision at the end of one graph-resident inner PCG iteration, exactly the
// host loop's: breakdown (p.Ap <= 0 or not finite) stops without counting the
// iteration; otherwise it is counted and the loop continues while
// ||r|| > thr and the budget allows.  scal[7] = p.Ap, scal[8] = r.r,
// scal[11] = thr; st[0] = iterations done, st[1] = budget, st[2] = breakdown.
__global__ void k_inner_cond(cudaGraphConditionalHandle h, const double* __restrict__ scal,
                             int* __restrict__ st) {
  const double pap = scal[7], rr = scal[8], thr = scal[11];
  if (!(pap > 0.0) || !isfinite(pap)) {
    st[2] = 1;
    cudaGraphSetConditional(h, 0u);
    return;
  }
  const int k = st[0] + 1;
  st[0] = k;
  cudaGraphSetConditional(h, (!(sqrt(rr) <= thr) && k < st[1]) ? 1u : 0u);
}

// Captures iterations 2.. of inner_pcg<float> into a WHILE conditional node.
// All pointers the body uses (fine vectors, level buffers, scalars) live as
// long as the solver, so the graph is built once and replayed for every inner
// solve.  On any capture error the solver keeps the host-driven loop.
bool Solver::build_inner_graph() {
  if (ig_failed_) return false;
  if (ig_) return true;
  const Grid& g = fp_.g;
  const int64_t n = g.ndof;
  auto ig = std::make_unique<InnerGraph>();
  bool ok = cudaGraphCreate(&ig->graph, 0) == cudaSuccess;
  cudaGraphConditionalHandle h{};
  cudaGraph_t body = nullptr;
  if (ok)
    ok = cudaGraphConditionalHandleCreate(&h, ig->graph, 1u, cudaGraphCondAssignDefault) ==
         cudaSuccess;
  if (ok) {
    cudaGraphNodeParams cp{};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t node;
    ok = cudaGraphAddNode(&node, ig->graph, nullptr, nullptr, 0, &cp) == cudaSuccess;
    if (ok) body = cp.conditional.phGraph_out[0];
  }
  if (ok)
    ok = cudaStreamBeginCaptureToGraph(s_, body, nullptr, nullptr, 0,
                                       cudaStreamCaptureModeThreadLocal) == cudaSuccess;
  if (ok) {
    const int64_t l0 = kernel_launch_count();
    const int64_t m0 = lowp_matvecs_;
    bool cap_ok = true;
    try {
      pending_x_ = true;  // every body execution starts with the last one's x update
      float* z = vcycle<float>(rf_.p, scal_.p + 9, true);
      flush_x();
      launch_cg_update_p<float>(pf_.p, z, scal_.p + 9, scal_.p + 6, n, s_);
      TG_CUDA(cudaMemcpyAsync(scal_.p + 6, scal_.p + 9, sizeof(double), cudaMemcpyDeviceToDevice,
                              s_));
      int nb = 0;
      launch_fine_op<float>(kApply, g, fp_.mc, Ef_.p, fp_.kept.p, pf_.p, nullptr, nullptr, 0.0f,
                            apf_.p, part_.p, &nb, s_, fp_.kept_node.p);
      launch_sum_partials(part_.p, nb, scal_.p + 7, s_);
      launch_cg_update_r_f(rf_.p, apf_.p, scal_.p + 6, scal_.p + 7, n, part_.p, s_, invdiagf_.p,
                           float(omega_), t1f_.p);
      launch_sum_partials(part_.p, kRedBlocks, scal_.p + 8, s_);
      k_inner_cond<<<1, 1, 0, s_>>>(h, scal_.p, istate_.p);
      TG_LAUNCH_CHECK();
    } catch (const Error&) {
      cap_ok = false;
    }
    pending_x_ = false;
    side_joined_ = true;
    cudaGraph_t out = nullptr;
    const bool end_ok = cudaStreamEndCapture(s_, &out) == cudaSuccess;
    ig->body_launches = kernel_launch_count() - l0;
    add_kernel_launches(-ig->body_launches);  // captured, not launched
    lowp_matvecs_ = m0;
    ok = cap_ok && end_ok;
  }
  if (ok) ok = cudaGraphInstantiate(&ig->exec, ig->graph, 0) == cudaSuccess;
  if (!ok) {
    cudaGetLastError();  // clear a capture error; the host loop runs instead
    ig_failed_ = true;
    return false;
  }
  ig_ = std::move(ig);
  return true;
}

template <>
bool Solver::inner_pcg<float>(int max_it, double rel_tol, SolverStats& st, int* iters) {
  const Grid& g = fp_.g;
  const int64_t n = g.ndof;
  launch_fill<float>(xf_.p, 0.0f, n, s_);
  TG_CUDA(cudaMemcpyAsync(rf_.p, zf_.p, size_t(n) * sizeof(float), cudaMemcpyDeviceToDevice, s_));
  launch_dot_f(rf_.p, rf_.p, n, part_.p, scal_.p + 10, s_);
  float* z = vcycle<float>(rf_.p, scal_.p + 6);
  TG_CUDA(cudaMemcpyAsync(pf_.p, z, size_t(n) * sizeof(float), cudaMemcpyDeviceToDevice, s_));
  const double b2 = read_scalar(10);
  const double thr = rel_tol * std::sqrt(b2);
  int nb = 0;
  *iters = 0;
  for (int k = 1; k <= max_it; ++k) {
    launch_fine_op<float>(kApply, g, fp_.mc, Ef_.p, fp_.kept.p, pf_.p, nullptr, nullptr, 0.0f,
                          apf_.p, part_.p, &nb, s_, fp_.kept_node.p);
    ++lowp_matvecs_;
    launch_sum_partials(part_.p, nb, scal_.p + 7, s_);
    // r now; x += alpha p when p is next overwritten or at exit (flush_x), or on
    // the side stream beside the next V-cycle's coarse levels (fork_x).
    launch_cg_update_r_f(rf_.p, apf_.p, scal_.p + 6, scal_.p + 7, n, part_.p, s_, invdiagf_.p,
                         float(omega_), t1f_.p);
    pending_x_ = true;
    launch_sum_partials(part_.p, kRedBlocks, scal_.p + 8, s_);
    double sc[2];
    read_scalars(7, 2, sc);
    if (!(sc[0] > 0.0) || !std::isfinite(sc[0])) {  // breakdown: alpha = 0, x and r untouched
      flush_x();
      ++st.inner_breakdowns;
      return k > 1;
    }
    *iters = k;
    if (std::sqrt(sc[1]) <= thr) {
      flush_x();
      return true;
    }
    if (k == 1 && max_it > 1 && use_graph_ && build_inner_graph()) {
      // Iterations 2.. on the device: one graph launch, one read-back.
      h_scal_[11] = thr;
      h_ist_[0] = 1;
      h_ist_[1] = max_it;
      h_ist_[2] = 0;
      TG_CUDA(cudaMemcpyAsync(scal_.p + 11, h_scal_ + 11, sizeof(double), cudaMemcpyHostToDevice,
                              s_));
      TG_CUDA(cudaMemcpyAsync(istate_.p, h_ist_, 3 * sizeof(int), cudaMemcpyHostToDevice, s_));
      TG_CUDA(cudaGraphLaunch(ig_->exec, s_));
      pending_x_ = true;  // the last body execution's x update
      flush_x();
      TG_CUDA(cudaMemcpyAsync(h_ist_, istate_.p, 3 * sizeof(int), cudaMemcpyDeviceToHost, s_));
      TG_CUDA(cudaStreamSynchronize(s_));
      const int done = h_ist_[0], broke = h_ist_[2];
      const int64_t runs = int64_t(done - 1) + broke;  // body executions
      add_kernel_launches(runs * ig_->body_launches);
      lowp_matvecs_ += 3 * runs;
      *iters = done;
      if (broke) ++st.inner_breakdowns;
      return true;
    }
    z = vcycle<float>(rf_.p, scal_.p + 9, true);
    flush_x();
    launch_cg_update_p<float>(pf_.p, z, scal_.p + 9, scal_.p + 6, n, s_);
    TG_CUDA(cudaMemcpyAsync(scal_.p + 6, scal_.p + 9, sizeof(double), cudaMemcpyDeviceToDevice, s_));
  }
  flush_x();
  (void)st;
  return true;
}

// Mixed precision: FP64 iterative refinement around FP32 MG-PCG inner solves.
// Convergence is judged on the FP64-recomputed residual ||b - A x|| <= tol ||b||.
// r = b - A x on the kept DOFs for the mixed loop.  In double-float arithmetic
// (tg_df.h) by default: the result agrees with the FP64 operator's to ~1e-14 of
// the operator's terms, far inside what the FP64 convergence test resolves, at a
// fraction of the FP64 pipe's time.
void Solver::refinement_residual() {
  const Grid& g = fp_.g;
  if (df_residual_) {
    launch_fine_residual_df(g, fp_.mc, E_, fp_.kept.p, x_.p, rhs_.p, r_.p, s_);
  } else {
    launch_fine_op<double>(kResidual, g, fp_.mc, E_, fp_.kept.p, x_.p, rhs_.p, nullptr, 0.0, r_.p,
                           nullptr, nullptr, s_);
  }
  ++fine_matvecs_;
}

bool Solver::mixed_refine(double tol, int max_it, bool warm, SolverStats& st) {
  mixed_partial_ = false;
  const Grid& g = fp_.g;
  const int64_t n = g.ndof;
  launch_dot(rhs_.p, rhs_.p, n, part_.p, scal_.p + 4, s_);
  const double bnorm2 = read_scalar(4);
  st.iterations = 0;
  st.residual = 0.0;
  if (!(bnorm2 > 0.0)) {
    launch_fill<double>(x_.p, 0.0, n, s_);
    return true;
  }
  const double bnorm = std::sqrt(bnorm2), threshold = tol * bnorm;
  if (warm) {
    launch_fine_op<double>(kResidual, g, fp_.mc, E_, fp_.kept.p, x_.p, rhs_.p, nullptr, 0.0, r_.p,
                           nullptr, nullptr, s_);
    ++fine_matvecs_;
  } else {
    launch_fill<double>(x_.p, 0.0, n, s_);
    TG_CUDA(cudaMemcpyAsync(r_.p, rhs_.p, size_t(n) * sizeof(double), cudaMemcpyDeviceToDevice, s_));
  }
  // Default: the inner FP32 solve targets 0.3x the reduction still needed, down
  // to 1e-5 -- one refinement usually finishes a warm-started solve, so the FP64
  // residual (FP64-bound, ~20x an FP32 apply) runs twice per solve, not three
  // times.  A recursive FP32 residual reaches 1e-5 whatever the true one does;
  // when the FP64 residual shows it fell short, another refinement follows.
  const double inner_tol = opt_.inner_tolerance > 0.0 ? opt_.inner_tolerance : 1e-5;
  const int max_ref = opt_.max_refinements > 0 ? opt_.max_refinements : 20;
  int total_inner = 0;
  double rn0 = -1.0;
  for (int ref = 0; ref <= max_ref; ++ref) {
    launch_dot(r_.p, r_.p, n, part_.p, scal_.p + 5, s_);
    const double rr = read_scalar(5);
    const double rn = std::sqrt(rr);
    st.residual = rn / bnorm;
    if (!std::isfinite(rn)) return false;
    if (rn <= threshold) {
      st.iterations = total_inner;
      return true;
    }
    if (rn0 < 0.0) rn0 = rn;
    if (ref == max_ref || total_inner >= max_it) {
      // Out of budget: x is finite and, when it reduced the residual, a better
      // start for the FP64 retry than its initial guess.
      mixed_partial_ = rn < rn0;
      break;
    }
    launch_scale_d2f(zf_.p, r_.p, scal_.p + 5, n, s_);
    int it = 0;
    // Default inner tolerance: 0.3x the reduction still needed, within
    // [1e-5, 0.1].
    const double itol = opt_.inner_tolerance > 0.0 ? inner_tol
                                                   : std::min(0.1, std::max(inner_tol, 0.3 * threshold / rn));
    inner_pcg<float>(std::min(budget_, max_it - total_inner), itol, st, &it);
    total_inner += it;
    launch_axpy_scaled_f2d(x_.p, xf_.p, scal_.p + 5, n, s_);
    refinement_residual();
    ++st.refinements;
  }
  st.iterations = total_inner;
  return false;
}

// ------------------------------------------------------------ Jacobi-PCG
// The Eigen-style Jacobi-PCG of mf_cg_solve (matfree.cpp:841-1076): squared
// threshold tol^2 |b|^2 clamped to DBL_MIN, the converging iteration uncounted.
bool Solver::jacobi_pcg(double tol, int max_it, bool warm, SolverStats& st) {
  const Grid& g = fp_.g;
  const int64_t n = g.ndof;
  const int maxIters = max_it > 0 ? max_it : int(std::min<int64_t>(2 * fp_.ng, 1 << 30));
  launch_dot(rhs_.p, rhs_.p, n, part_.p, scal_.p + 4, s_);
  const double rhs2 = read_scalar(4);
  st.iterations = 0;
  st.residual = 0.0;
  if (rhs2 == 0.0) {
    launch_fill<double>(x_.p, 0.0, n, s_);
    return true;
  }
  double threshold = tol * tol * rhs2;
  if (threshold < std::numeric_limits<double>::min()) threshold = std::numeric_limits<double>::min();
  if (!warm) launch_fill<double>(x_.p, 0.0, n, s_);
  launch_fine_op<double>(kResidual, g, fp_.mc, E_, fp_.kept.p, x_.p, rhs_.p, nullptr, 0.0, r_.p,
                         nullptr, nullptr, s_);
  ++fine_matvecs_;
  launch_dot(r_.p, r_.p, n, part_.p, scal_.p + 2, s_);
  double rr = read_scalar(2);
  if (rr < threshold) {
    st.residual = std::sqrt(rr / rhs2);
    return st.residual <= tol;
  }
  launch_scale_mask(p_.p, r_.p, invdiag_.p, n, part_.p, s_);
  launch_sum_partials(part_.p, kRedBlocks, scal_.p + 0, s_);
  int i = 0, nb = 0;
  while (i < maxIters) {
    launch_fine_op<double>(kApply, g, fp_.mc, E_, fp_.kept.p, p_.p, nullptr, nullptr, 0.0, ap_.p,
                           part_.p, &nb, s_);
    ++fine_matvecs_;
    launch_sum_partials(part_.p, nb, scal_.p + 1, s_);
    launch_cg_update_xr<double>(x_.p, r_.p, p_.p, ap_.p, scal_.p + 0, scal_.p + 1, n, part_.p, s_);
    launch_sum_partials(part_.p, kRedBlocks, scal_.p + 2, s_);
    rr = read_scalar(2);
    if (rr < threshold) break;
    launch_scale_mask(z_.p, r_.p, invdiag_.p, n, part_.p, s_);
    launch_sum_partials(part_.p, kRedBlocks, scal_.p + 3, s_);
    launch_cg_update_p<double>(p_.p, z_.p, scal_.p + 3, scal_.p + 0, n, s_);
    TG_CUDA(cudaMemcpyAsync(scal_.p + 0, scal_.p + 3, sizeof(double), cudaMemcpyDeviceToDevice, s_));
    ++i;
  }
  st.iterations = i;
  st.residual = std::sqrt(rr / rhs2);
  launch_dot(x_.p, x_.p, n, part_.p, scal_.p + 5, s_);
  const bool finite = std::isfinite(read_scalar(5));
  return st.residual <= tol && finite;
}

// ------------------------------------------------------------------ solve
SolverStats Solver::solve(double tol, int max_it, const double* guess, double* u) {
  SolverStats st;
  const double t0 = now_ms();
  fine_matvecs_ = lowp_matvecs_ = 0;
  const Grid& g = fp_.g;
  st.hier_built = have_mg_ && numeric_ok_;
  st.t_mg_build_ms = mg_build_ms_;
  if (fp_.ng == 0) {
    st.converged = true;
    launch_mask_select(u, nullptr, fp_.up.p, fp_.kept.p, g.ndof, s_);
    TG_CUDA(cudaStreamSynchronize(s_));
    return st;
  }
  const int cap = max_it > 0 ? max_it : int(std::max<int64_t>(1000, 2 * fp_.ng));
  const bool warm = guess != nullptr;
  auto seed = [&]() { launch_mask_select(x_.p, guess, nullptr, fp_.kept.p, g.ndof, s_); };
  bool solved = false;
  if (have_mg_ && numeric_ok_) {
    if (mixed_) {
      // The mixed form's inner FP32 iterations are budgeted at 3x the MG budget:
      // each refinement restarts CG (about 1.3x the iterations of one FP64 run)
      // and an FP32 iteration costs about 1/6 of the FP64 retry's.
      if (warm) seed();
      solved = mixed_refine(tol, std::min(cap, 3 * budget_), warm, st);
    }
    if (mixed_ && l1_tc_) {
      // A tensor-core completion wait that ran out is a device error, not a
      // solver verdict.
      int tc_err = 0;
      TG_CUDA(cudaMemcpyAsync(&tc_err, tc_err_.p, sizeof(int), cudaMemcpyDeviceToHost, s_));
      TG_CUDA(cudaStreamSynchronize(s_));
      if (tc_err)
        raise(TG_EDEVICE, "level-1 tensor-core operator: MMA completion wait timed out");
    }
    if (mixed_ && !solved) st.mixed_fallback = true;
    if (!solved && (!mixed_ || build_numeric<double>())) {
      // The FP64 retry of a mixed solve starts from the mixed attempt's last
      // iterate when that attempt made progress (high-contrast designs can need
      // more FP32 refinements than the budget allows while each one still
      // gains); otherwise from the caller's guess or zero.
      const bool resume = mixed_ && mixed_partial_;
      if (warm && !resume) seed();
      solved = mgpcg(tol, std::min(cap, budget_), warm || resume, st);
    }
    st.mg_cycles = st.iterations;
    if (solved) {
      st.used_mg = true;
      st.mg_levels = levels();
    }
  }
  if (!solved) {
    if (warm) seed();
    solved = jacobi_pcg(tol, cap, warm, st);
    st.used_mg = false;
    st.mg_levels = 0;
  }
  st.converged = solved;
  st.matvecs = fine_matvecs_;
  st.matvecs_lowp = lowp_matvecs_;
  if (solved) launch_mask_select(u, x_.p, fp_.up.p, fp_.kept.p, g.ndof, s_);
  TG_CUDA(cudaStreamSynchronize(s_));
  st.t_solve_ms = now_ms() - t0;
  return st;
}

}  // namespace tg
