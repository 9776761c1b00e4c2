// api.cu -- the extern "C" boundary (include/topopt_gb300.h) and the resident
// SIMP job.  Host code above the kernels: argument validation with the
// reference's messages, the optimizer loop of simp_optimize
// (core/src/simp/simp.cpp:2018-2592) and the OC bisection of oc_update
// (simp.cpp:948-1025).
//
// OC bisection parity.  The reference compares a SEQUENTIAL FP64 sum of the
// filtered candidate against the target (simp.cpp:1003-1016).  Here the volume
// is summed exactly (192-bit fixed point, order independent).  The sequential
// sum s differs from the exact sum S by at most gamma_{n-1} * S (n terms, all
// non-negative), so when |S - target| exceeds that bound the branch is the
// reference's for certain; otherwise the filtered candidate is copied to the
// host and summed sequentially in grid order, exactly as the reference does.
// With the candidate and the filter rounding like the reference (k_simp.cu),
// every bisection branch -- and therefore x_new -- is bit-identical.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "tg_solver.h"

namespace tg {

namespace {
thread_local std::string g_err;
int g_device = 0;
std::atomic<int64_t> g_launches{0};

double now_ms() {
  return std::chrono::duration<double, std::milli>(
             std::chrono::steady_clock::now().time_since_epoch())
      .count();
}
}  // namespace

void raise(int code, const std::string& msg) { throw Error(code, msg); }

namespace {
thread_local cudaStream_t t_alloc_stream = nullptr;
std::mutex g_pin_mu;
std::vector<char*> g_pin_free;  // free 256-byte pinned slots
bool g_pool_tuned[64] = {};
}  // namespace

cudaStream_t alloc_stream() { return t_alloc_stream; }

AllocScope::AllocScope(cudaStream_t s) : prev(t_alloc_stream) {
  t_alloc_stream = s;
  // Keep freed blocks in the device pool for the next job instead of returning
  // them to the system at every synchronisation (process-local pool setting).
  int dev = 0;
  if (cudaGetDevice(&dev) == cudaSuccess && dev >= 0 && dev < 64) {
    std::lock_guard<std::mutex> lk(g_pin_mu);
    if (!g_pool_tuned[dev]) {
      cudaMemPool_t pool;
      if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
        uint64_t keep = ~uint64_t(0);
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
      }
      g_pool_tuned[dev] = true;
    }
  }
}
AllocScope::~AllocScope() { t_alloc_stream = prev; }

void* pinned_scalars(size_t bytes) {
  if (bytes > 256) raise(TG_EINVAL, "pinned_scalars: request above 256 bytes");
  std::lock_guard<std::mutex> lk(g_pin_mu);
  if (g_pin_free.empty()) {
    void* slab = nullptr;
    TG_CUDA(cudaMallocHost(&slab, 64 * 256));  // kept for the life of the process
    for (int i = 0; i < 64; ++i) g_pin_free.push_back(static_cast<char*>(slab) + 256 * i);
  }
  char* p = g_pin_free.back();
  g_pin_free.pop_back();
  return p;
}

void pinned_release(void* p) {
  if (!p) return;
  std::lock_guard<std::mutex> lk(g_pin_mu);
  g_pin_free.push_back(static_cast<char*>(p));
}
int device_ordinal() { return g_device; }
void set_last_error(const std::string& msg) { g_err = msg; }
namespace {
thread_local int64_t t_launches = 0;  // this thread's launches (graph capture accounting)
}
void note_launch() {
  g_launches.fetch_add(1, std::memory_order_relaxed);
  ++t_launches;
}
int64_t kernel_launch_count() { return t_launches; }
void add_kernel_launches(int64_t delta) { g_launches.fetch_add(delta, std::memory_order_relaxed); }

void cuda_fail(cudaError_t e, const char* what, const char* file, int line) {
  char buf[512];
  std::snprintf(buf, sizeof buf, "CUDA error %d (%s) in %s at %s:%d", int(e), cudaGetErrorString(e),
                what, file, line);
  throw Error(e == cudaErrorMemoryAllocation ? TG_ENOMEM : TG_EDEVICE, buf);
}

template <class F>
int guarded(F&& fn, bool device = true) {
  try {
    if (device) TG_CUDA(cudaSetDevice(g_device));
    fn();
    return TG_OK;
  } catch (const Error& e) {
    g_err = e.what();
    return e.code;
  } catch (const std::bad_alloc&) {
    g_err = "host allocation failed";
    return TG_ENOMEM;
  } catch (const std::exception& e) {
    g_err = e.what();
    return TG_EINVAL;
  }
}

// A stream that lives for one call.
struct CallStream {
  cudaStream_t s = nullptr;
  CallStream() { TG_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking)); }
  ~CallStream() {
    if (s) cudaStreamDestroy(s);
  }
};

template <class T>
void upload(DBuf<T>& d, const T* h, size_t n, cudaStream_t s) {
  d.alloc(n);
  TG_CUDA(cudaMemcpyAsync(d.p, h, n * sizeof(T), cudaMemcpyHostToDevice, s));
}

void validate_grid(const tg_grid* g) {
  if (!g) raise(TG_EINVAL, "grid is null");
  if (g->nx < 1 || g->ny < 1 || g->nz < 1) raise(TG_EINVAL, "grid dimensions must be >= 1");
  if (!(g->spacing > 0.0)) raise(TG_EINVAL, "grid spacing must be > 0");
  if (int64_t(g->nx + 1) * (g->ny + 1) * (g->nz + 1) * 3 > (int64_t(1) << 31) - 1)
    raise(TG_EINVAL, "grid too large: DOF indices must fit a 32-bit int");
}

// SimpParams checks (simp.cpp:34-41).
void validate_params(const tg_simp_params* p) {
  if (!p) raise(TG_EINVAL, "params is null");
  if (!(p->youngs_modulus > 0.0)) raise(TG_EINVAL, "simp: youngs_modulus (E0) must be > 0");
  if (!(p->penalty > 0.0)) raise(TG_EINVAL, "simp: penalty (p) must be > 0");
  if (!(p->density_min > 0.0 && p->density_min <= 1.0))
    raise(TG_EINVAL, "simp: density_min must be in (0, 1]");
  if (p->material_law != 0 && p->material_law != 1)
    raise(TG_EINVAL, "simp: material_law must be 0 (reference) or 1 (modified)");
  if (p->material_law == 1 && !(p->e_min > 0.0 && p->e_min < p->youngs_modulus))
    raise(TG_EINVAL, "simp: e_min must be in (0, E0) for the modified law");
}

// effective_design_mask (simp.cpp:2610-2633): Empty voxels -> FrozenVoid (2),
// Load (4) and Fixture (5) voxels -> FrozenSolid (1), the caller's entry
// elsewhere.  Mask bytes are MaskValue (voxel.hpp:42-46): 0 Active, 1 FrozenSolid,
// 2 FrozenVoid; any other byte is rejected.
std::vector<uint8_t> effective_mask(const tg_grid* g, const uint8_t* mask, const char* who) {
  if (!mask) raise(TG_EINVAL, std::string(who) + ": mask size != voxel_count");
  const int64_t nv = int64_t(g->nx) * g->ny * g->nz;
  std::vector<uint8_t> eff(static_cast<size_t>(nv));
  for (int64_t e = 0; e < nv; ++e) {
    if (mask[e] > 2)
      raise(TG_EINVAL, std::string(who) +
                           ": mask values must be 0 (Active), 1 (FrozenSolid) or 2 (FrozenVoid)");
    const uint8_t t = g->tags ? g->tags[e] : uint8_t(1);
    eff[size_t(e)] = t == 0 ? uint8_t(2) : ((t == 4 || t == 5) ? uint8_t(1) : mask[e]);
  }
  return eff;
}

tg_solve_options default_solve(const tg_solve_options* o) {
  tg_solve_options d;
  std::memset(&d, 0, sizeof d);
  if (o) d = *o;
  if (d.solver != TG_SOLVER_MGCG && d.solver != TG_SOLVER_JACOBI_CG)
    raise(TG_EINVAL, "solve options: unknown solver kind");
  if (d.precision != TG_PREC_FP64 && d.precision != TG_PREC_MIXED)
    raise(TG_EINVAL, "solve options: unknown precision");
  if (d.precision == TG_PREC_MIXED && d.solver != TG_SOLVER_MGCG)
    raise(TG_EINVAL, "solve options: mixed precision needs the multigrid solver");
  if (d.coarsening < TG_COARSEN_DEFAULT || d.coarsening > TG_COARSEN_ALIGNED)
    raise(TG_EINVAL, "solve options: unknown coarsening");
  if (d.graph_mode != TG_GRAPH_ON && d.graph_mode != TG_GRAPH_OFF)
    raise(TG_EINVAL, "solve options: unknown graph_mode");
  if (d.smooth_sweeps < 0 || d.smooth_sweeps > 8)
    raise(TG_EINVAL, "solve options: smooth_sweeps must be in [0, 8]");
  if (d.mixed_residual != TG_RESIDUAL_DF && d.mixed_residual != TG_RESIDUAL_FP64)
    raise(TG_EINVAL, "solve options: unknown mixed_residual");
  if (d.coarse_smoother < TG_SMOOTHER_AUTO || d.coarse_smoother > TG_SMOOTHER_CHEBYSHEV)
    raise(TG_EINVAL, "solve options: unknown coarse_smoother");
  return d;
}

void fill_info(tg_cg_info* info, const SolverStats& st, const FineProblem& fp, double t_build,
               double t_total) {
  if (!info) return;
  std::memset(info, 0, sizeof *info);
  info->converged = st.converged;
  info->iterations = st.iterations;
  info->residual = st.residual;
  info->used_multigrid = st.used_mg;
  info->mg_levels = st.mg_levels;
  info->hier_built = st.hier_built;
  info->mg_cycles_attempted = st.mg_cycles;
  info->matvecs = st.matvecs;
  info->matvecs_lowp = st.matvecs_lowp;
  info->refinements = st.refinements;
  info->ng = int32_t(fp.ng);
  info->mixed_fallback = st.mixed_fallback;
  info->inner_breakdowns = st.inner_breakdowns;
  info->t_build_ms = t_build;
  info->t_mg_build_ms = st.t_mg_build_ms;
  info->t_solve_ms = st.t_solve_ms;
  info->t_total_ms = t_total;
}

// ------------------------------------------------------------ filter state
struct FilterState {
  FilterStencil st;
  DBuf<unsigned char> st_buf;
  const void* st_dev = nullptr;
  DBuf<double> hs, tmp;
  void init(const Grid& g, double radius, const uint8_t* act, cudaStream_t s) {
    if (!(radius > 0.0)) raise(TG_EINVAL, "make_density_filter: radius must be > 0");
    st = FilterStencil::make(radius);
    st_dev = filter_stencil_device(st, st_buf, s);
    hs.alloc(size_t(g.nv));
    tmp.alloc(size_t(g.nv));
    launch_weight_sum(g, st_dev, st.n, act, hs.p, s);
  }
  void fwd(const Grid& g, const uint8_t* act, const double* x, double* out, cudaStream_t s) {
    launch_filter_fwd(g, st_dev, st.n, act, hs.p, x, out, s);
  }
  void adj(const Grid& g, const uint8_t* act, const double* x, double* out, cudaStream_t s) {
    launch_filter_adj(g, st_dev, st.n, act, hs.p, x, tmp.p, out, s);
  }
  size_t bytes() const { return st_buf.bytes() + hs.bytes() + tmp.bytes(); }
};

// ------------------------------------------------------------ OC update
// Candidate fields of one projected bisection pass: up to kOcMulti, at most
// 128 MB of them.
int projected_candidates(int64_t nv) {
  const int64_t cap = (int64_t(128) << 20) / (8 * std::max<int64_t>(nv, 1));
  return int(std::max<int64_t>(1, std::min<int64_t>(kOcMulti, cap)));
}

struct OcState {
  // sq, lo, hi and dvd carry double-float pairs for the fast volume pass (the
  // projected update reuses sq and lo as FP64 scratch).
  DBuf<double> dcf, dvf, xp, sq, lo, hi, dvd, vpart, vsum;
  int fast_evals = 0, exact_evals = 0;
  double radius = 1.5;
  DBuf<uint64_t> part, total;
  DBuf<int> inexact;
  uint64_t* h_total = nullptr;  // pinned: 3 limbs + flag
  std::vector<double> h_xp;
  double* h_v = nullptr;  // pinned: kOcMulti candidate volumes
  int64_t n_solid = 0;
  int fallbacks = 0, evals = 0, passes = 0;
  bool carry = false;  // oc_update_masked: voxels outside the design set keep x
  // Projected bisection: kproj candidate fields evaluated per pass.
  DBuf<double> cand;
  int kproj = 0;
  void init_projected(const Grid& g) {
    if (kproj > 0) return;
    kproj = projected_candidates(g.nv);
    cand.alloc(size_t(kproj) * size_t(g.nv));
  }
  void init(const Grid& g, cudaStream_t) {
    for (DBuf<double>* d : {&dcf, &dvf, &xp, &sq, &lo, &hi, &dvd}) d->alloc(size_t(g.nv));
    vpart.alloc(size_t(kRedBlocks) * kOcMulti);
    vsum.alloc(kOcMulti);
    h_v = static_cast<double*>(pinned_scalars(kOcMulti * sizeof(double)));
    part.alloc(size_t(3 * exact_sum_blocks()));
    total.alloc(3);
    inexact.alloc(1);
    h_total = static_cast<uint64_t*>(pinned_scalars(4 * sizeof(uint64_t)));
  }
  ~OcState() {
    pinned_release(h_total);
    pinned_release(h_v);
  }
  size_t bytes() const {
    return dcf.bytes() + dvf.bytes() + xp.bytes() + sq.bytes() + lo.bytes() + hi.bytes() +
           dvd.bytes() + vpart.bytes() + vsum.bytes() + part.bytes() + total.bytes() + inexact.bytes() +
           cand.bytes();
  }
};

// Exact sum of v over the active voxels, as a double (3 roundings of the exact
// 192-bit value); *exact tells whether every term was representable.
double exact_volume(OcState& oc, const Grid& g, const uint8_t* act, const double* v, bool* exact,
                    cudaStream_t s) {
  TG_CUDA(cudaMemsetAsync(oc.inexact.p, 0, sizeof(int), s));
  launch_exact_sum(v, act, g.nv, oc.part.p, oc.total.p, oc.inexact.p, s);
  TG_CUDA(cudaMemcpyAsync(oc.h_total, oc.total.p, 3 * sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
  TG_CUDA(cudaMemcpyAsync(oc.h_total + 3, oc.inexact.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  TG_CUDA(cudaStreamSynchronize(s));
  *exact = (reinterpret_cast<const int*>(oc.h_total + 3)[0] == 0);
  return double(oc.h_total[2]) + std::ldexp(double(oc.h_total[1]), -64) +
         std::ldexp(double(oc.h_total[0]), -128);
}

// phys_vol(candidate) > target, decided exactly as the reference's sequential
// sum would decide it (see the file comment).
bool volume_exceeds(OcState& oc, const Grid& g, const uint8_t* act,
                    const std::vector<uint8_t>& act_h, double target, cudaStream_t s) {
  bool exact = false;
  const double S = exact_volume(oc, g, act, oc.xp.p, &exact, s);
  if (exact && std::isfinite(S)) {
    const double u = std::ldexp(1.0, -53);
    const double n1 = double(std::max<int64_t>(oc.n_solid - 1, 0));
    const double gamma = n1 * u / (1.0 - n1 * u);
    const double bound = gamma * S * 1.0000001 + 8.0 * u * S + 1e-300;
    if (S - target > bound) return true;
    if (target - S > bound) return false;
  }
  ++oc.fallbacks;
  oc.h_xp.resize(size_t(g.nv));
  TG_CUDA(cudaMemcpyAsync(oc.h_xp.data(), oc.xp.p, size_t(g.nv) * sizeof(double),
                          cudaMemcpyDeviceToHost, s));
  TG_CUDA(cudaStreamSynchronize(s));
  double v = 0.0;
  for (int64_t e = 0; e < g.nv; ++e)
    if (act_h[size_t(e)]) v += oc.h_xp[size_t(e)];
  return v > target;
}

// oc_update (simp.cpp:948-1025) on device-resident fields; dvf must hold the
// filtered unit volume sensitivity.  Each bisection branch is first decided from
// the fast linear volume sum_n dv_n x~_n(lambda) (k_oc_volume), whose distance to
// the reference's sequential sum of filtered candidates is bounded by
//   (n - 1) u V            (the sequential sum)
// + (m + 1) u V            (the filter's m products and the division, per voxel)
// + (m + 1) u V            (the rounding of dv itself)
// + 12 u V                 (candidate: reference div/mul/sqrt vs sqrt(B)/sqrt(lambda))
// + (n/(608*256) + 64) u V (this FP64 sum: a per-thread run, then trees),
// m the stencil size, u = 2^-53.  Only inside that band is the exact path run:
// the reference's candidate, the filter and the exact sum, then -- if still
// within the sequential-sum bound -- the host's sequential sum.
void oc_update_device(OcState& oc, FilterState& fs, const Grid& g, const uint8_t* act,
                      const std::vector<uint8_t>& act_h, const double* x, const double* dc,
                      double volfrac, double move, double rho_min, double* xnew, cudaStream_t s) {
  fs.adj(g, act, dc, oc.dcf.p, s);
  const double target = volfrac * double(oc.n_solid);
  launch_oc_prepare(x, oc.dcf.p, oc.dvf.p, act, g.nv, move, rho_min, oc.sq.p, oc.lo.p, oc.hi.p,
                    oc.dvd.p, s);
  const double u = std::ldexp(1.0, -53);
  const double n = double(std::max<int64_t>(oc.n_solid, 1));
  const double m = double(fs.st.n);
  // + 8192 u: the fast pass runs in double-float arithmetic -- the split of its
  // four FP64 inputs (2^-49 each), the product, clamp and accumulation (~2^-46
  // relative per operation over a per-thread run of a few dozen terms) -- far
  // below the n u of the reference's own sequential sum.
  const double eps =
      (n + 2.0 * (m + 1.0) + 12.0 + n / (double(kRedBlocks) * 256.0) + 64.0 + 8192.0) * u * 1.01;
  // Fast volumes are computed ahead, kmax lambdas per pass over the fields: the
  // next doublings while bracketing, the next levels of the bisection tree
  // (breadth first) while bisecting.  Every branch is still decided one at a
  // time, in the reference's order, from the volume of exactly the lambda the
  // sequential loop would test, so the speculation changes no decision.  A
  // candidate costs a few FP64 operations per voxel: on large grids the pass is
  // FP64-bound, and 4 per pass (two bisection levels and one more midpoint)
  // wastes less work than 16 (four levels, of which one path is used).
  const int kmax = g.nv > (int64_t(1) << 20) ? 4 : kOcMulti;
  std::vector<std::pair<double, double>> known;  // (lambda, fast volume)
  auto lookup = [&](double lam, double* V) {
    for (const auto& kv : known)
      if (kv.first == lam) {
        *V = kv.second;
        return true;
      }
    return false;
  };
  auto batch = [&](const std::vector<double>& lams) {
    OcCands cs;
    cs.k = int(std::min<size_t>(lams.size(), size_t(kmax)));
    for (int k = 0; k < cs.k; ++k) cs.c[k] = 1.0 / std::sqrt(lams[size_t(k)]);
    launch_oc_volume_multi(oc.sq.p, oc.lo.p, oc.hi.p, oc.dvd.p, g.nv, cs, oc.vpart.p, oc.vsum.p,
                           s);
    TG_CUDA(cudaMemcpyAsync(oc.h_v, oc.vsum.p, sizeof(double) * cs.k, cudaMemcpyDeviceToHost, s));
    TG_CUDA(cudaStreamSynchronize(s));
    ++oc.passes;
    for (int k = 0; k < cs.k; ++k) known.emplace_back(lams[size_t(k)], oc.h_v[k]);
  };
  auto eval = [&](double lam) {
    ++oc.evals;
    double V = 0.0;
    if (!lookup(lam, &V)) {
      batch({lam});
      lookup(lam, &V);
    }
    const double bound = eps * V / (1.0 - eps) + 1e-300;
    if (std::isfinite(V)) {
      if (V - target > bound) {
        ++oc.fast_evals;
        return true;
      }
      if (target - V > bound) {
        ++oc.fast_evals;
        return false;
      }
    }
    ++oc.exact_evals;
    launch_oc_candidate(x, oc.dcf.p, oc.dvf.p, act, g.nv, lam, move, rho_min, oc.carry, xnew, s);
    fs.fwd(g, act, xnew, oc.xp.p, s);
    return volume_exceeds(oc, g, act, act_h, target, s);
  };
  double l1 = 0.0, l2 = 1.0;
  double Vtmp = 0.0;
  while (l2 < 1e30) {
    if (!lookup(l2, &Vtmp)) {
      std::vector<double> c;
      for (double t = l2; int(c.size()) < kmax && t < 1e30; t *= 2.0) c.push_back(t);
      batch(c);
    }
    if (!eval(l2)) break;
    l2 *= 2.0;
  }
  for (int it = 0; it < 100 && (l2 - l1) > 1e-6 * (l1 + l2); ++it) {
    const double lmid = 0.5 * (l1 + l2);
    if (!lookup(lmid, &Vtmp)) {
      // The midpoints the next bisection steps can reach, breadth first,
      // computed with the loop's own arithmetic.
      std::vector<double> c;
      std::vector<std::pair<double, double>> lv{{l1, l2}};
      while (!lv.empty() && int(c.size()) < kmax) {
        std::vector<std::pair<double, double>> nx;
        for (const auto& iv : lv) {
          if (int(c.size()) >= kmax) break;
          const double m = 0.5 * (iv.first + iv.second);
          c.push_back(m);
          nx.emplace_back(iv.first, m);
          nx.emplace_back(m, iv.second);
        }
        lv.swap(nx);
      }
      batch(c);
    }
    if (eval(lmid))
      l1 = lmid;
    else
      l2 = lmid;
  }
  launch_oc_candidate(x, oc.dcf.p, oc.dvf.p, act, g.nv, 0.5 * (l1 + l2), move, rho_min, oc.carry,
                      xnew, s);
}

// oc_update_projected (simp.cpp:1665-1726) on device-resident fields: the
// projection derivative at xtilde chained before the filter transpose (dproj and
// dc * dproj staged in sq and lo, which the projected update does not otherwise
// use), then the reference's bracketing and bisection, every branch decided by
// the projected volume sum_e heaviside_project(filter(x_new(lambda)))_e over the
// design voxels.  The volumes of up to kproj multipliers come from one pass
// (the next doublings while bracketing, the next bisection levels' midpoints
// while bisecting); each branch is still decided one at a time, in the
// reference's order, from the volume of exactly the multiplier it tests.  The
// projection uses the device's tanh, so a volume can differ from the host's in
// the last bits and a branch on a near-tie may go the other way: this form is
// held to the reference within tolerance, not bit for bit.
void oc_update_projected_device(OcState& oc, FilterState& fs, const Grid& g, const uint8_t* act,
                                const double* x, const double* xtilde, const double* dc,
                                double beta, double eta, double volfrac, double move,
                                double rho_min, double* xnew, cudaStream_t s) {
  oc.init_projected(g);
  launch_proj_chain(xtilde, dc, act, g.nv, beta, eta, oc.sq.p, oc.lo.p, s);
  fs.adj(g, act, oc.lo.p, oc.dcf.p, s);
  fs.adj(g, act, oc.sq.p, oc.dvf.p, s);
  const double target = volfrac * double(oc.n_solid);
  std::vector<std::pair<double, double>> known;  // (lambda, projected volume)
  auto lookup = [&](double lam, double* V) {
    for (const auto& kv : known)
      if (kv.first == lam) {
        *V = kv.second;
        return true;
      }
    return false;
  };
  auto batch = [&](const std::vector<double>& lams) {
    ProjLambdas ls;
    ls.k = int(std::min<size_t>(lams.size(), size_t(oc.kproj)));
    for (int k = 0; k < ls.k; ++k) ls.lam[k] = lams[size_t(k)];
    launch_oc_candidates_projected(x, oc.dcf.p, oc.dvf.p, act, g.nv, ls, move, rho_min, oc.carry,
                                   oc.cand.p, s);
    launch_proj_volume(g, fs.st_dev, fs.st.n, act, fs.hs.p, oc.cand.p, ls.k, beta, eta,
                       oc.vpart.p, oc.vsum.p, s);
    TG_CUDA(cudaMemcpyAsync(oc.h_v, oc.vsum.p, sizeof(double) * ls.k, cudaMemcpyDeviceToHost, s));
    TG_CUDA(cudaStreamSynchronize(s));
    ++oc.passes;
    for (int k = 0; k < ls.k; ++k) known.emplace_back(ls.lam[k], oc.h_v[k]);
  };
  auto exceeds = [&](double lam) {
    ++oc.evals;
    double V = 0.0;
    if (!lookup(lam, &V)) {
      batch({lam});
      lookup(lam, &V);
    }
    return V > target;
  };
  double l1 = 0.0, l2 = 1.0, Vtmp = 0.0;
  while (l2 < 1e30) {
    if (!lookup(l2, &Vtmp)) {
      std::vector<double> c;
      for (double t = l2; int(c.size()) < oc.kproj && t < 1e30; t *= 2.0) c.push_back(t);
      batch(c);
    }
    if (!exceeds(l2)) break;
    l2 *= 2.0;
  }
  for (int it = 0; it < 100 && (l2 - l1) > 1e-6 * (l1 + l2); ++it) {
    const double lmid = 0.5 * (l1 + l2);
    if (!lookup(lmid, &Vtmp)) {
      // Midpoints of the next bisection levels, breadth first, as many as one
      // pass holds (the loop's own arithmetic).
      std::vector<double> c;
      std::vector<std::pair<double, double>> lv{{l1, l2}};
      while (!lv.empty() && int(c.size()) < oc.kproj) {
        std::vector<std::pair<double, double>> nx;
        for (const auto& iv : lv) {
          if (int(c.size()) >= oc.kproj) break;
          const double m = 0.5 * (iv.first + iv.second);
          c.push_back(m);
          nx.emplace_back(iv.first, m);
          nx.emplace_back(m, iv.second);
        }
        lv.swap(nx);
      }
      batch(c);
    }
    if (exceeds(lmid))
      l1 = lmid;
    else
      l2 = lmid;
  }
  ProjLambdas last;
  last.k = 1;
  last.lam[0] = 0.5 * (l1 + l2);
  launch_oc_candidates_projected(x, oc.dcf.p, oc.dvf.p, act, g.nv, last, move, rho_min, oc.carry,
                                 xnew, s);
}

// mma_update / mma_update_masked (simp.cpp:1433-1489, :2736-2784) with the
// subproblem of mma_update_joint (mma_joint.cpp) on device-resident fields: dc
// through the filter transpose (bit-exact), the fixed dv, the coefficients and
// box (bit-exact per voxel), g0 = the exact sum of the filtered design over the
// design set minus the target, and the dual's doubling and bisection to
// 1e-9 (1 + l1 + l2), up to kOcMulti multipliers per pass, each branch decided
// in the reference's order.  The dual sums are fixed-order device sums, not the
// reference's sequential ones, so a branch on a near-tie may differ: this
// updater is held to the reference within tolerance.
void mma_update_device(OcState& oc, FilterState& fs, const Grid& g, const uint8_t* act,
                       MmaFields& m, int iter, DBuf<uint64_t>& scale, const double* x,
                       const double* xphys, const double* dc, double volfrac, double move,
                       double rho_min, double* xnew, cudaStream_t s) {
  fs.adj(g, act, dc, oc.dcf.p, s);
  bool exact = false;
  const double vol = exact_volume(oc, g, act, xphys, &exact, s);
  const double g0 = vol - volfrac * double(oc.n_solid);
  launch_mma_prepare(m, x, oc.dcf.p, oc.dvf.p, act, g.nv, iter, move, rho_min, scale.p,
                     oc.vpart.p, oc.vsum.p, s);
  TG_CUDA(cudaMemcpyAsync(oc.h_v, oc.vsum.p, sizeof(double), cudaMemcpyDeviceToHost, s));
  TG_CUDA(cudaStreamSynchronize(s));
  const double b = -g0 + oc.h_v[0];
  std::vector<std::pair<double, double>> known;  // (lambda, constraint sum)
  auto lookup = [&](double lam, double* v) {
    for (const auto& kv : known)
      if (kv.first == lam) {
        *v = kv.second;
        return true;
      }
    return false;
  };
  const int kmax = g.nv > (int64_t(1) << 22) ? 4 : kOcMulti;
  auto batch = [&](const std::vector<double>& lams) {
    ProjLambdas ls;
    ls.k = int(std::min<size_t>(lams.size(), size_t(kmax)));
    for (int k = 0; k < ls.k; ++k) ls.lam[k] = lams[size_t(k)];
    launch_mma_dual(m, act, g.nv, ls, oc.vpart.p, oc.vsum.p, s);
    TG_CUDA(cudaMemcpyAsync(oc.h_v, oc.vsum.p, sizeof(double) * ls.k, cudaMemcpyDeviceToHost, s));
    TG_CUDA(cudaStreamSynchronize(s));
    ++oc.passes;
    for (int k = 0; k < ls.k; ++k) known.emplace_back(ls.lam[k], oc.h_v[k]);
  };
  auto positive = [&](double lam) {  // gval(candidate(lam)) > 0
    ++oc.evals;
    double v = 0.0;
    if (!lookup(lam, &v)) {
      batch({lam});
      lookup(lam, &v);
    }
    return (v - b) > 0.0;
  };
  // lambda = 0 and the first doublings in one pass.
  {
    std::vector<double> c{0.0};
    for (double t = 1.0; int(c.size()) < kmax; t *= 2.0) c.push_back(t);
    batch(c);
  }
  double lambda = 0.0, tmp = 0.0;
  if (positive(0.0)) {
    double l1 = 0.0, l2 = 1.0;
    while (l2 < 1e30) {
      if (!lookup(l2, &tmp)) {
        std::vector<double> c;
        for (double t = l2; int(c.size()) < kmax && t < 1e30; t *= 2.0) c.push_back(t);
        batch(c);
      }
      if (!positive(l2)) break;
      l2 *= 2.0;
    }
    for (int it = 0; it < 100 && (l2 - l1) > 1e-9 * (1.0 + l1 + l2); ++it) {
      const double lmid = 0.5 * (l1 + l2);
      if (!lookup(lmid, &tmp)) {
        std::vector<double> c;
        std::vector<std::pair<double, double>> lv{{l1, l2}};
        while (!lv.empty() && int(c.size()) < kmax) {
          std::vector<std::pair<double, double>> nx;
          for (const auto& iv : lv) {
            if (int(c.size()) >= kmax) break;
            const double mm = 0.5 * (iv.first + iv.second);
            c.push_back(mm);
            nx.emplace_back(iv.first, mm);
            nx.emplace_back(mm, iv.second);
          }
          lv.swap(nx);
        }
        batch(c);
      }
      if (positive(lmid))
        l1 = lmid;
      else
        l2 = lmid;
    }
    lambda = 0.5 * (l1 + l2);
  }
  launch_mma_candidate(m, act, g.nv, lambda, xnew, s);
  // xold2 = xold1; xold1 = x.
  std::swap(m.xold1, m.xold2);
  TG_CUDA(cudaMemcpyAsync(m.xold1, x, size_t(g.nv) * sizeof(double), cudaMemcpyDeviceToDevice, s));
}

}  // namespace tg

using namespace tg;

// ------------------------------------------------------------------ the job
struct tg_job {
  // Declared first, destroyed last: every buffer below is allocated
  // stream-ordered on this stream and freed on it before it goes.
  struct OwnedStream {
    cudaStream_t s = nullptr;
    ~OwnedStream() {
      if (s) cudaStreamDestroy(s);
    }
  } owned;
  cudaStream_t s = nullptr;
  tg_simp_params params{};
  tg_simp_options opt{};
  FineProblem fp;
  std::unique_ptr<Solver> solver;
  FilterState filt;
  OcState oc;
  DBuf<uint8_t> solid;          // the design set: solid voxels, or Active voxels (masked)
  std::vector<uint8_t> solid_h;
  bool masked = false;          // the masked overload (simp.cpp:2989-3640)
  DBuf<uint8_t> eff;            // effective design mask (masked jobs)
  std::vector<uint8_t> eff_h;
  DBuf<double> x, xnew, xphys, E, u, dc, part, scal;
  // The projection plan (simp.cpp:1053-1068); empty for the unprojected loop.
  std::vector<tg_projection_stage> stages;
  double eta = 0.5;
  int stage = 0;        // the stage the next steps run
  DBuf<double> xtilde;  // filter(x), before the projection (projected jobs)
  bool projecting() const { return !stages.empty(); }
  // MMA (updater == TG_UPDATER_MMA): the run's asymptotes, last two designs and
  // the subproblem's fields.
  bool mma = false;
  int mma_iter = 0;
  DBuf<double> mma_buf;  // 10 fields of nv
  DBuf<uint64_t> mma_scale;
  MmaFields mf{};
  double* h_scal = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr, evf = nullptr;
  int64_t n_solid = 0;
  int iteration = 0;
  bool xphys_valid = false;
  std::vector<double> hist_c;
  std::vector<int> hist_cg;
  // The active domain (ActiveDomainRun, simp.cpp:1745-1766): the resolved band,
  // the one-way latch and its record, the running fraction mean, the band the
  // previous armed solve ran under (device), the analysis grid's tags, BCs and
  // loads (to build the restricted system), and the restricted system with its
  // solver, rebuilt only when the mask changes.
  struct ActiveDomain {
    int band = 0;
    bool latched = false, have_prev = false;
    int latch_iteration = 0, hot_streak = 0;
    int64_t escape_count = 0, n_solid = 0;
    double fraction_sum = 0.0;
    int64_t fraction_count = 0;
    std::string reason;
    tg_grid grid{};
    std::vector<uint8_t> tags_h, cur_h, built_h;
    std::vector<tg_dirichlet_bc> bcs;
    std::vector<tg_nodal_load> loads;
    DBuf<uint8_t> tags, prev, cur, tmp;
    DBuf<unsigned long long> count;
    FineProblem fp;
    std::unique_ptr<Solver> solver;  // declared after fp: destroyed first
    bool armed() const { return band > 0 && !latched; }
    void record(double f) {
      fraction_sum += f;
      ++fraction_count;
    }
    // The latch is one way: the restricted system is not solved again, so its
    // device memory goes back (stream-ordered) when the mask is switched off.
    void release_restricted() {
      solver.reset();
      fp = FineProblem{};
      built_h.clear();
      built_h.shrink_to_fit();
      cur_h.clear();
      cur_h.shrink_to_fit();
    }
    size_t bytes() const {
      return tags.bytes() + prev.bytes() + cur.bytes() + tmp.bytes() + count.bytes() +
             fp.device_bytes() + (solver ? solver->device_bytes() : 0);
    }
  } ad;

  ~tg_job() {
    ad.solver.reset();
    solver.reset();
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (evf) cudaEventDestroy(evf);
    pinned_release(h_scal);
  }
  size_t bytes() const {
    size_t b = fp.device_bytes() + filt.bytes() + oc.bytes() + solid.bytes() + eff.bytes();
    for (const DBuf<double>* d : {&x, &xnew, &xphys, &E, &u, &dc, &part, &scal, &xtilde, &mma_buf})
      b += d->bytes();
    return b + (solver ? solver->device_bytes() : 0) + ad.bytes();
  }
};

namespace tg {
namespace {

// Job setup.  With a mask (the masked overload, simp.cpp:3017-3072): the
// effective mask, the analysis grid with FrozenVoid voxels made Empty, the
// Active-only filter and design set, and the start design Active = volfrac,
// FrozenSolid = 1, else 0.
void job_init(tg_job* j, const tg_grid* grid, const tg_simp_params* params,
              const tg_dirichlet_bc* bcs, int nbc, const tg_nodal_load* loads, int nloads,
              const tg_simp_options* options, const uint8_t* mask = nullptr) {
  validate_grid(grid);
  validate_params(params);
  if (!options) raise(TG_EINVAL, "options is null");
  const tg_simp_options& o = *options;
  if (!(o.volume_fraction > 0.0 && o.volume_fraction <= 1.0))
    raise(TG_EINVAL, "simp_optimize: volume_fraction must be in (0, 1]");
  if (!(o.move > 0.0)) raise(TG_EINVAL, "simp_optimize: move must be > 0");
  if (o.max_iterations < 1) raise(TG_EINVAL, "simp_optimize: max_iterations must be >= 1");
  if (o.change_tol < 0.0) raise(TG_EINVAL, "simp_optimize: change_tol must be >= 0");
  if (!(o.filter_radius > 0.0)) raise(TG_EINVAL, "make_density_filter: radius must be > 0");
  if (!(o.cg_tolerance > 0.0)) raise(TG_EINVAL, "simp_optimize: cg_tolerance must be > 0");
  // validate_projection_options (simp.cpp:59-74).
  if (o.projection_stages < 0 || (o.projection_stages > 0 && !o.projection))
    raise(TG_EINVAL, "simp_optimize: projection must hold projection_stages stages");
  if (o.projection_stages > 0) {
    if (!(o.projection_eta > 0.0 && o.projection_eta < 1.0))
      raise(TG_EINVAL, "simp_optimize: projection_eta must be in (0, 1)");
    for (int i = 0; i < o.projection_stages; ++i) {
      const tg_projection_stage& ps = o.projection[i];
      if (!(ps.beta > 0.0) || !std::isfinite(ps.beta))
        raise(TG_EINVAL, "simp_optimize: projection stage beta must be finite and > 0");
      if (!(ps.move > 0.0)) raise(TG_EINVAL, "simp_optimize: projection stage move must be > 0");
      if (ps.iterations < 1)
        raise(TG_EINVAL, "simp_optimize: projection stage iterations must be >= 1");
    }
    j->stages.assign(o.projection, o.projection + o.projection_stages);
    j->eta = o.projection_eta;
  }
  if (o.updater != TG_UPDATER_OC && o.updater != TG_UPDATER_MMA)
    raise(TG_EINVAL, "simp_optimize: updater must be TG_UPDATER_OC or TG_UPDATER_MMA");
  // validate_updater_options (simp.cpp:83-88).
  if (o.updater == TG_UPDATER_MMA && o.projection_stages > 0)
    raise(TG_EINVAL, "simp_optimize: MMA updater does not support a Heaviside projection "
                     "schedule; use OC or clear options.projection");
  j->mma = o.updater == TG_UPDATER_MMA;
  j->params = *params;
  j->opt = o;
  j->opt.projection = nullptr;  // the job keeps its own copy of the plan
  j->opt.solve = default_solve(&o.solve);
  TG_CUDA(cudaStreamCreateWithFlags(&j->owned.s, cudaStreamNonBlocking));
  j->s = j->owned.s;
  TG_CUDA(cudaEventCreate(&j->ev0));
  TG_CUDA(cudaEventCreate(&j->ev1));
  TG_CUDA(cudaEventCreate(&j->evf));
  cudaStream_t s = j->s;
  AllocScope scope(s);
  tg_grid analysis = *grid;
  std::vector<uint8_t> atags;
  j->masked = mask != nullptr;
  if (j->masked) {
    j->eff_h = effective_mask(grid, mask, "simp_optimize");
    atags.resize(j->eff_h.size());
    for (size_t e = 0; e < atags.size(); ++e)
      atags[e] = j->eff_h[e] == 2 ? uint8_t(0) : (grid->tags ? grid->tags[e] : uint8_t(1));
    analysis.tags = atags.data();
  }
  j->fp.build(analysis, params->poisson, bcs, nbc, loads, nloads, nullptr, s);
  const Grid& g = j->fp.g;
  j->solver = std::make_unique<Solver>(j->fp, j->opt.solve, s);
  if (j->masked) {
    j->solid_h.resize(j->eff_h.size());
    for (size_t e = 0; e < j->eff_h.size(); ++e) j->solid_h[e] = j->eff_h[e] == 0;
    upload(j->eff, j->eff_h.data(), j->eff_h.size(), s);
  } else {
    j->solid_h = j->fp.elem_h;  // no mask on this path: the design set is the solid set
  }
  j->n_solid = 0;
  for (uint8_t v : j->solid_h) j->n_solid += v;
  upload(j->solid, j->solid_h.data(), j->solid_h.size(), s);
  // resolve_active_domain_band (simp.cpp:1773-1782): < 0 is the auto band.
  j->ad.band = o.active_domain_band < 0 ? tg_active_domain_auto_band(o.filter_radius)
                                        : o.active_domain_band;
  if (j->ad.band > 0) {
    tg_job::ActiveDomain& ad = j->ad;
    ad.grid = analysis;
    if (analysis.tags) {
      ad.tags_h.assign(analysis.tags, analysis.tags + g.nv);
      ad.grid.tags = ad.tags_h.data();
      upload(ad.tags, ad.tags_h.data(), ad.tags_h.size(), s);
    }
    ad.bcs.assign(bcs, bcs + nbc);
    ad.loads.assign(loads, loads + nloads);
    for (uint8_t v : j->fp.elem_h) ad.n_solid += v;  // solid voxels of the analysis grid
    for (DBuf<uint8_t>* d : {&ad.prev, &ad.cur, &ad.tmp}) d->alloc(size_t(g.nv));
    ad.count.alloc(1);
  }
  for (DBuf<double>* d : {&j->x, &j->xnew, &j->xphys, &j->E, &j->dc}) d->alloc(size_t(g.nv));
  if (j->projecting()) j->xtilde.alloc(size_t(g.nv));
  if (j->mma) {
    const size_t n = size_t(g.nv);
    j->mma_buf.alloc(10 * n);
    j->mma_scale.alloc(1);
    TG_CUDA(cudaMemsetAsync(j->mma_buf.p, 0, j->mma_buf.bytes(), s));
    double* b = j->mma_buf.p;
    j->mf = MmaFields{b, b + n, b + 2 * n, b + 3 * n, b + 4 * n,
                      b + 5 * n, b + 6 * n, b + 7 * n, b + 8 * n, b + 9 * n};
  }
  j->u.alloc(size_t(g.ndof));
  j->part.alloc(size_t(4 * kRedBlocks + 152 * 32));
  j->scal.alloc(8);
  j->h_scal = static_cast<double*>(pinned_scalars(8 * sizeof(double)));
  j->filt.init(g, o.filter_radius, j->solid.p, s);
  j->oc.init(g, s);
  j->oc.n_solid = j->n_solid;
  j->oc.carry = j->masked;
  // dv = filter_sensitivity(ones on solid voxels) (simp.cpp:967-976): fixed.
  std::vector<double> ones(size_t(g.nv));
  for (int64_t e = 0; e < g.nv; ++e) ones[size_t(e)] = j->solid_h[size_t(e)] ? 1.0 : 0.0;
  TG_CUDA(cudaMemcpyAsync(j->xnew.p, ones.data(), j->xnew.bytes(), cudaMemcpyHostToDevice, s));
  j->filt.adj(g, j->solid.p, j->xnew.p, j->oc.dvf.p, s);
  // simp_uniform_density (simp.cpp:305-312); masked: simp.cpp:3066-3072.
  for (int64_t e = 0; e < g.nv; ++e) {
    ones[size_t(e)] = j->solid_h[size_t(e)] ? o.volume_fraction : 0.0;
    if (j->masked && j->eff_h[size_t(e)] == 1) ones[size_t(e)] = 1.0;
  }
  if (o.initial_design) {
    // warm_start_design (simp.cpp:324-344): the seed's mean over the design set
    // (summed in voxel order, on the host, as the reference sums it) rescaled to
    // the target, each design entry clamped to [density_min, 1], one pass of the
    // loop's filter; masked jobs then pin FrozenSolid to 1 and every other
    // non-Active voxel to 0 (simp.cpp:3083-3090).
    const double* seed = o.initial_design;
    double sum = 0.0;
    int64_t n = 0;
    for (int64_t e = 0; e < g.nv; ++e)
      if (j->solid_h[size_t(e)]) {
        sum += seed[e];
        ++n;
      }
    const double mean = n > 0 ? sum / double(n) : 0.0;
    const double rho_min = params->density_min;
    for (int64_t e = 0; e < g.nv; ++e) {
      double v = 0.0;
      if (j->solid_h[size_t(e)]) {
        if (mean > 1e-12) {
          const double scale = o.volume_fraction / mean;
          v = std::min(1.0, std::max(rho_min, scale * seed[e]));
        } else {
          v = o.volume_fraction;
        }
      }
      ones[size_t(e)] = v;
    }
    TG_CUDA(cudaMemcpyAsync(j->xnew.p, ones.data(), j->xnew.bytes(), cudaMemcpyHostToDevice, s));
    j->filt.fwd(g, j->solid.p, j->xnew.p, j->x.p, s);
    if (j->masked) launch_mask_pins(j->eff.p, g.nv, j->x.p, s);
  } else {
    TG_CUDA(cudaMemcpyAsync(j->x.p, ones.data(), j->x.bytes(), cudaMemcpyHostToDevice, s));
  }
  TG_CUDA(cudaStreamSynchronize(s));
  j->opt.initial_design = nullptr;  // consumed; the caller's buffer need not outlive the call
}

double read1(tg_job* j, const double* dptr) {
  TG_CUDA(cudaMemcpyAsync(j->h_scal, dptr, sizeof(double), cudaMemcpyDeviceToHost, j->s));
  TG_CUDA(cudaStreamSynchronize(j->s));
  return j->h_scal[0];
}

// Compliance + dc at the current physical density and displacement, over the
// elements of the system that was solved (`elem`: the job's solid set, or the
// restricted set of an active-domain solve, whose other elements get no energy
// and no sensitivity, simp.cpp:752-763).
double job_sensitivity(tg_job* j, const uint8_t* elem = nullptr) {
  const Grid& g = j->fp.g;
  const tg_simp_params& p = j->params;
  int nparts = 0;
  // The mixed form evaluates element energies in double-float (~1e-14), the
  // plain form in FP64 as the reference does.
  launch_sensitivity(g, j->fp.mc, j->xphys.p, elem ? elem : j->fp.elem.p, j->u.p,
                     p.youngs_modulus, p.penalty, p.density_min, p.material_law, p.e_min,
                     j->dc.p, j->part.p, &nparts, j->s,
                     j->opt.solve.precision == TG_PREC_MIXED);
  launch_sum_partials(j->part.p, nparts, j->scal.p, j->s);
  return read1(j, j->scal.p);
}

// Penalised solve at the current physical density.
SolverStats job_solve(tg_job* j, double tol, int max_it) {
  AllocScope scope(j->s);  // lazily built state (FP64 fallback hierarchy) is the job's
  const Grid& g = j->fp.g;
  const tg_simp_params& p = j->params;
  launch_modulus(j->xphys.p, j->fp.elem.p, g.nv, p.youngs_modulus, p.penalty, p.density_min,
                 p.material_law, p.e_min, j->E.p, j->s);
  j->solver->set_modulus(j->E.p);
  return j->solver->solve(tol, max_it, nullptr, j->u.p);
}

// One trajectory solve under the active domain (active_domain_solve,
// simp.cpp:1809-1896).  Armed: the escape check against the previous band
// (first escape: latch, full domain), then the mask of the current physical
// density, the restricted system (rebuilt when the mask changed) and its solve;
// a restricted system that fails its void gates or does not converge latches
// the mask off and the same field is re-solved on the full domain.  After a
// restricted solve the fraction latch counts iterations at >= 0.85
// (kActiveDomainLatchFraction / kActiveDomainLatchWindow, simp.hpp:363-364).
// *af: the active fraction of the solve that ran (1 on the full domain);
// *elem: its element set.
SolverStats ad_job_solve(tg_job* j, double tol, int max_it, double* af, const uint8_t** elem) {
  tg_job::ActiveDomain& ad = j->ad;
  *af = 1.0;
  *elem = j->fp.elem.p;
  if (ad.armed()) {
    AllocScope scope(j->s);
    const Grid& g = j->fp.g;
    const tg_simp_params& p = j->params;
    const int iteration = j->iteration + 1;
    const uint8_t* tags = ad.tags.p;  // null: every voxel solid, nothing pinned
    int64_t esc = 0;
    if (ad.have_prev) {
      launch_active_domain_escape(tags, j->xphys.p, ad.prev.p, p.density_min, g.nv, ad.count.p,
                                  j->s);
      unsigned long long n = 0;
      TG_CUDA(cudaMemcpyAsync(&n, ad.count.p, sizeof n, cudaMemcpyDeviceToHost, j->s));
      TG_CUDA(cudaStreamSynchronize(j->s));
      esc = int64_t(n);
    }
    if (esc > 0) {
      ad.latched = true;
      ad.latch_iteration = iteration;
      ad.escape_count = esc;
      ad.release_restricted();
      char buf[192];
      std::snprintf(buf, sizeof buf,
                    "escape detected: %lld element(s) took material outside the active band "
                    "(growth invariant failed); mask disabled, full domain restored",
                    static_cast<long long>(esc));
      ad.reason = buf;
      ad.record(1.0);
    } else {
      launch_active_domain_mask(g.nx, g.ny, g.nz, tags, j->xphys.p, p.density_min, ad.band,
                                ad.cur.p, ad.tmp.p, ad.count.p, j->s);
      unsigned long long active = 0;
      ad.cur_h.resize(size_t(g.nv));
      TG_CUDA(cudaMemcpyAsync(ad.cur_h.data(), ad.cur.p, size_t(g.nv), cudaMemcpyDeviceToHost,
                              j->s));
      TG_CUDA(cudaMemcpyAsync(&active, ad.count.p, sizeof active, cudaMemcpyDeviceToHost, j->s));
      TG_CUDA(cudaStreamSynchronize(j->s));
      const double fraction = ad.n_solid > 0 ? double(active) / double(ad.n_solid) : 1.0;
      try {
        if (!ad.solver || ad.cur_h != ad.built_h) {
          ad.solver.reset();
          ad.built_h.clear();
          ad.fp.build(ad.grid, p.poisson, ad.bcs.data(), int(ad.bcs.size()), ad.loads.data(),
                      int(ad.loads.size()), ad.cur_h.data(), j->s);
          ad.solver = std::make_unique<Solver>(ad.fp, j->opt.solve, j->s);
          ad.built_h = ad.cur_h;
        }
        launch_modulus(j->xphys.p, ad.fp.elem.p, g.nv, p.youngs_modulus, p.penalty,
                       p.density_min, p.material_law, p.e_min, j->E.p, j->s);
        ad.solver->set_modulus(j->E.p);
        const SolverStats st = ad.solver->solve(tol, max_it, nullptr, j->u.p);
        if (!st.converged)
          raise(TG_ENONCONV, "CG did not reach the requested tolerance within max_iterations");
        *af = fraction;
        *elem = ad.fp.elem.p;
        ad.record(fraction);
        if (fraction >= 0.85) {
          if (++ad.hot_streak >= 5) {
            ad.latched = true;
            ad.latch_iteration = iteration;
            // This solve's u and element set are read by the sensitivity that
            // follows; the restricted system is released at the next solve.
            char buf[192];
            std::snprintf(buf, sizeof buf,
                          "active fraction >= %.2f for %d consecutive iterations (band covers "
                          "the domain and buys nothing)",
                          0.85, 5);
            ad.reason = buf;
          }
        } else {
          ad.hot_streak = 0;
        }
        std::swap(ad.prev, ad.cur);
        ad.have_prev = true;
        return st;
      } catch (const Error& e) {
        // The reference catches every exception of the restricted solve; device
        // faults are not the band's doing and stay fatal here.
        if (e.code == TG_EDEVICE) throw;
        ad.latched = true;
        ad.latch_iteration = iteration;
        ad.reason = std::string("restricted solve failed: fea_solve_mgcg_matfree: ") + e.what();
        ad.record(1.0);
        ad.release_restricted();
      }
    }
  } else if (ad.band > 0) {
    ad.record(1.0);  // latched: still counted, as 1.0
    if (ad.solver) ad.release_restricted();  // latched on the fraction last iteration
  }
  return job_solve(j, tol, max_it);
}

// xPhys = filter(x), projected on the design voxels at the current stage's beta
// when projecting (simp.cpp:2197-2199, :3200-3203), then the mask pins.  Volume
// sums run over the design set only, which the pins never touch, so they see
// the unpinned field as the reference's active_volfrac does.
void job_filter_x(tg_job* j) {
  const Grid& g = j->fp.g;
  if (j->projecting()) {
    j->filt.fwd(g, j->solid.p, j->x.p, j->xtilde.p, j->s);
    launch_project(j->xtilde.p, j->solid.p, g.nv, j->stages[size_t(j->stage)].beta, j->eta,
                   j->xphys.p, nullptr, j->s);
  } else {
    j->filt.fwd(g, j->solid.p, j->x.p, j->xphys.p, j->s);
  }
  if (j->masked) launch_mask_pins(j->eff.p, g.nv, j->xphys.p, j->s);
  j->xphys_valid = true;
}

// One design iteration of simp_optimize's loop body (simp.cpp:2158-2340).
int job_step(tg_job* j, tg_simp_iteration* row) {
  AllocScope scope(j->s);
  const Grid& g = j->fp.g;
  const tg_simp_options& o = j->opt;
  tg_simp_iteration r;
  std::memset(&r, 0, sizeof r);
  const double t0 = now_ms();
  TG_CUDA(cudaEventRecord(j->ev0, j->s));
  if (!j->xphys_valid) job_filter_x(j);
  TG_CUDA(cudaEventRecord(j->evf, j->s));  // filter time from events, no host wait here
  const double t1 = now_ms();
  double af = 1.0;
  const uint8_t* elem = nullptr;
  SolverStats st = ad_job_solve(j, o.cg_tolerance, o.cg_max_iterations, &af, &elem);
  const double t2 = now_ms();
  if (!st.converged) {
    Error e(TG_ENONCONV, "simp_optimize: the trajectory solve did not reach the requested tolerance");
    e.iterations = st.iterations;
    e.residual = st.residual;
    throw e;
  }
  const double c = job_sensitivity(j, elem);
  const double t3 = now_ms();
  const int fb0 = j->oc.evals, ps0 = j->oc.passes, ex0 = j->oc.exact_evals,
            hf0 = j->oc.fallbacks;
  double beta = 0.0;
  if (j->projecting()) {
    // xtilde = filter(x) is current: job_filter_x ran for this x.
    const tg_projection_stage& ps = j->stages[size_t(j->stage)];
    beta = ps.beta;
    oc_update_projected_device(j->oc, j->filt, g, j->solid.p, j->x.p, j->xtilde.p, j->dc.p,
                               ps.beta, j->eta, o.volume_fraction, ps.move,
                               j->params.density_min, j->xnew.p, j->s);
  } else if (j->mma) {
    mma_update_device(j->oc, j->filt, g, j->solid.p, j->mf, ++j->mma_iter, j->mma_scale,
                      j->x.p, j->xphys.p, j->dc.p, o.volume_fraction, o.move,
                      j->params.density_min, j->xnew.p, j->s);
  } else {
    oc_update_device(j->oc, j->filt, g, j->solid.p, j->solid_h, j->x.p, j->dc.p,
                     o.volume_fraction, o.move, j->params.density_min, j->xnew.p, j->s);
  }
  launch_absdiff_max(j->xnew.p, j->x.p, g.nv, j->part.p, j->scal.p + 1, j->s);
  const double change = read1(j, j->scal.p + 1);
  std::swap(j->x.p, j->xnew.p);
  job_filter_x(j);
  bool exact = false;
  const double vol = exact_volume(j->oc, g, j->solid.p, j->xphys.p, &exact, j->s);
  TG_CUDA(cudaEventRecord(j->ev1, j->s));
  TG_CUDA(cudaEventSynchronize(j->ev1));
  float dev_ms = 0.0f, filt_ms = 0.0f;
  TG_CUDA(cudaEventElapsedTime(&dev_ms, j->ev0, j->ev1));
  TG_CUDA(cudaEventElapsedTime(&filt_ms, j->ev0, j->evf));
  const double t4 = now_ms();
  j->iteration += 1;
  r.iteration = j->iteration;
  r.compliance = c;
  r.change = change;
  r.volume_fraction = j->n_solid > 0 ? vol / double(j->n_solid) : 0.0;
  r.cg_iterations = st.iterations;
  r.mg_levels = st.mg_levels;
  r.used_multigrid = st.used_mg;
  r.oc_volume_evals = j->oc.evals - fb0;
  r.oc_volume_passes = j->oc.passes - ps0;
  r.t_filter_ms = filt_ms;
  r.t_solve_ms = t2 - t1;
  r.t_sensitivity_ms = t3 - t2;
  r.t_update_ms = t4 - t3;
  r.t_total_ms = t4 - t0;
  r.t_device_ms = dev_ms;
  r.fine_matvecs = st.matvecs;
  r.fine_matvecs_lowp = st.matvecs_lowp;
  r.beta = beta;
  r.hier_built = st.hier_built ? 1 : 0;
  r.mg_cycles_attempted = st.mg_cycles;
  r.oc_exact_evals = j->oc.exact_evals - ex0;
  r.oc_host_fallbacks = j->oc.fallbacks - hf0;
  r.active_fraction = af;
  j->hist_c.push_back(c);
  j->hist_cg.push_back(st.iterations);
  if (row) *row = r;
  return TG_OK;
}

// rung_infeasible (simp.cpp:1140-1186) at the SimpOptions defaults
// (simp.hpp:1299-1302): ratio 100, CG blow-up 4, flat 1e-3, window 5.
bool rung_infeasible(const std::vector<double>& c, const std::vector<int>& cg) {
  const int window = 5;
  const int n = int(c.size());
  if (n < window + 1) return false;
  if (!(std::isfinite(c[0]) && c[0] > 0.0)) return false;
  int cgmin = cg[0];
  for (int i = 1; i < n - window; ++i) cgmin = std::min(cgmin, cg[size_t(i)]);
  if (cgmin <= 0) return false;
  const double cbar = 100.0 * c[0], cgbar = 4.0 * double(cgmin);
  double lo = c[size_t(n - window)], hi = lo;
  for (int i = n - window; i < n; ++i) {
    if (!std::isfinite(c[size_t(i)])) return false;
    if (!(c[size_t(i)] >= cbar)) return false;
    if (!(double(cg[size_t(i)]) >= cgbar)) return false;
    lo = std::min(lo, c[size_t(i)]);
    hi = std::max(hi, c[size_t(i)]);
  }
  if (!(lo > 0.0)) return false;
  return (hi - lo) / lo <= 1e-3;
}


// mma_objective_plateau (simp.cpp:1081-1134): the running-minimum improvement
// over the trailing window below tol, behind the min_drop progress gate with
// its flatness escape over min_flat_windows windows.
bool mma_objective_plateau(const std::vector<double>& c, const tg_simp_options& o) {
  const int window = o.mma_plateau_window;
  if (window <= 0) return false;
  const int n = int(c.size());
  if (n < window + 1) return false;
  double best_now = c[0];
  for (int i = 1; i < n; ++i) best_now = c[size_t(i)] < best_now ? c[size_t(i)] : best_now;
  const double min_drop = o.mma_plateau_min_drop, tol = o.mma_plateau_tol;
  if (min_drop > 0.0 && !(best_now <= c[0] * (1.0 - min_drop))) {
    bool escape = false;
    const int flat = o.mma_plateau_flat_windows;
    if (flat > 0 && n >= flat * window + 1) {
      double before = c[0];
      for (int i = 1; i < n - flat * window; ++i) before = c[size_t(i)] < before ? c[size_t(i)] : before;
      if (before > 0.0) escape = (before - best_now) / before < tol;
    }
    if (!escape) return false;
  }
  double best_prev = c[0];
  for (int i = 1; i < n - window; ++i) best_prev = c[size_t(i)] < best_prev ? c[size_t(i)] : best_prev;
  if (!(best_prev > 0.0)) return false;
  return (best_prev - best_now) / best_prev < tol;
}

// ------------------------------------------------------ strength analysis
void validate_strength(const tg_strength_spec* sp) {
  if (!sp) raise(TG_EINVAL, "strength spec is null");
  if (!(sp->printed_iso > 0.0 && sp->printed_iso < 1.0))
    raise(TG_EINVAL, "analyze_fixed_design: printed_iso must be in (0, 1)");
  const double* b = sp->build_dir;
  if (!(std::sqrt(b[0] * b[0] + b[1] * b[1] + b[2] * b[2]) >= 1e-12))
    raise(TG_EINVAL, "max_interlayer_tension: build_dir is zero length");
  if (!(std::isfinite(sp->yield_strength) && sp->yield_strength > 0.0))
    raise(TG_EINVAL, "stress margin: yield_strength_mpa must be finite and > 0");
  if (!(std::isfinite(sp->z_knockdown) && sp->z_knockdown > 0.0 && sp->z_knockdown <= 1.0))
    raise(TG_EINVAL, "stress margin: z_knockdown must be in (0, 1]");
}

// load_path_connected (voxelize.cpp:609-726): breadth-first flood fill over the
// printed voxels from the printed Fixture voxels, 26-connected; connected when
// every Load voxel is reached; vacuous without Load or Fixture voxels.
bool load_path_host(const Grid& g, const uint8_t* tags, const double* rho, double iso) {
  if (!tags) return true;
  int64_t nload = 0, nfix = 0;
  for (int64_t e = 0; e < g.nv; ++e) {
    nload += tags[e] == 4;
    nfix += tags[e] == 5;
  }
  if (nload == 0 || nfix == 0) return true;
  auto printed = [&](int64_t e) { return tags[e] != 0 && rho[e] > iso; };
  std::vector<uint8_t> seen(size_t(g.nv), 0);
  std::vector<int64_t> queue;
  int64_t reached = 0;
  for (int64_t e = 0; e < g.nv; ++e)
    if (tags[e] == 5 && printed(e)) {
      seen[size_t(e)] = 1;
      queue.push_back(e);
    }
  for (size_t h = 0; h < queue.size(); ++h) {
    const int64_t e = queue[h];
    reached += tags[e] == 4;
    const int i = int(e % g.nx), jj = int((e / g.nx) % g.ny), k = int(e / (int64_t(g.nx) * g.ny));
    for (int dk = -1; dk <= 1; ++dk)
      for (int dj = -1; dj <= 1; ++dj)
        for (int di = -1; di <= 1; ++di) {
          const int a = i + di, b = jj + dj, c = k + dk;
          if (a < 0 || b < 0 || c < 0 || a >= g.nx || b >= g.ny || c >= g.nz) continue;
          const int64_t q = (int64_t(c) * g.ny + b) * g.nx + a;
          if (seen[size_t(q)] || !printed(q)) continue;
          seen[size_t(q)] = 1;
          queue.push_back(q);
        }
  }
  return reached == nload;
}

// compute_stress_margin (report.cpp:464-491) and the scalar gate
// (gate_margin_effective, analyze.cpp:84-118).
void fill_margins(tg_fixed_design_analysis* a, const tg_strength_spec& sp) {
  const double inf = std::numeric_limits<double>::infinity();
  const double vm = a->max_von_mises, il = a->max_interlayer_tension;
  if (!(std::isfinite(vm) && vm >= 0.0))
    raise(TG_EINVAL, "stress margin: max_von_mises_stress must be finite and >= 0");
  if (!(std::isfinite(il) && il >= 0.0))
    raise(TG_EINVAL, "stress margin: max_interlayer_tension must be finite and >= 0");
  a->margin_in_plane = vm > 0.0 ? sp.yield_strength / vm : inf;
  a->margin_interlayer = il > 0.0 ? (sp.z_knockdown * sp.yield_strength) / il : inf;
  a->margin_worst_case = std::min(a->margin_in_plane, a->margin_interlayer);
  a->margin_effective = a->margin_worst_case * sp.infill_knockdown;
}

// analyze_fixed_design on a job built for the analysis grid: the density goes
// to xPhys, the certification solve at the job's tolerance, the stresses of the
// printed voxels with the solid modulus, the margins, the load-path belt and
// the gate.  rho_host is the same density on the host (for the belt).
void analyze_on_job(tg_job* aj, const double* rho_host, const uint8_t* tags,
                    const tg_strength_spec& sp, tg_fixed_design_analysis* out,
                    double* vm_out, double* stress_out, double* disp_out = nullptr) {
  AllocScope scope(aj->s);
  std::memset(out, 0, sizeof *out);
  const Grid& g = aj->fp.g;
  TG_CUDA(cudaMemcpyAsync(aj->xphys.p, rho_host, aj->xphys.bytes(), cudaMemcpyHostToDevice,
                          aj->s));
  aj->xphys_valid = true;
  const SolverStats st = job_solve(aj, aj->opt.cg_tolerance, aj->opt.cg_max_iterations);
  out->cg_iterations = st.iterations;
  if (!st.converged) {
    out->non_convergent = 1;  // never accepted (analyze.cpp:270-283)
    return;
  }
  out->compliance = job_sensitivity(aj);
  DBuf<uint64_t> peaks(3);
  DBuf<double> vm_d, sig_d;
  if (vm_out) vm_d.alloc(size_t(g.nv));
  if (stress_out) sig_d.alloc(size_t(6 * g.nv));
  TG_CUDA(cudaMemsetAsync(peaks.p, 0, 3 * sizeof(uint64_t), aj->s));
  launch_element_stress(g, aj->fp.elem.p, aj->xphys.p, aj->u.p, aj->params.youngs_modulus,
                        aj->params.poisson, g.h, sp.build_dir, sp.printed_iso, vm_d.p, sig_d.p,
                        peaks.p, aj->s);
  uint64_t h[3];
  TG_CUDA(cudaMemcpyAsync(h, peaks.p, sizeof h, cudaMemcpyDeviceToHost, aj->s));
  if (vm_out)
    TG_CUDA(cudaMemcpyAsync(vm_out, vm_d.p, vm_d.bytes(), cudaMemcpyDeviceToHost, aj->s));
  if (stress_out)
    TG_CUDA(cudaMemcpyAsync(stress_out, sig_d.p, sig_d.bytes(), cudaMemcpyDeviceToHost, aj->s));
  TG_CUDA(cudaStreamSynchronize(aj->s));
  double vm = 0.0, il = 0.0;
  std::memcpy(&vm, &h[0], sizeof vm);
  std::memcpy(&il, &h[1], sizeof il);
  out->max_von_mises = vm;
  out->max_interlayer_tension = il;
  out->printed_voxels = int64_t(h[2]);
  fill_margins(out, sp);
  out->load_path_ok = load_path_host(g, tags, rho_host, sp.printed_iso) ? 1 : 0;
  out->accepted = out->load_path_ok && out->margin_effective >= sp.margin_stop;
  if (disp_out) {
    // The displacement on printed nodes exactly as solved, 0 on nodes attached
    // only to non-printed voxels (analyze.cpp:385-394).
    TG_CUDA(cudaMemcpyAsync(disp_out, aj->u.p, aj->u.bytes(), cudaMemcpyDeviceToHost, aj->s));
    TG_CUDA(cudaStreamSynchronize(aj->s));
    std::vector<uint8_t> printed(size_t(g.nnodes), 0);
    for (int k = 0; k < g.nz; ++k)
      for (int j = 0; j < g.ny; ++j)
        for (int i = 0; i < g.nx; ++i) {
          const int64_t e = (int64_t(k) * g.ny + j) * g.nx + i;
          if ((tags && tags[e] == 0) || !(rho_host[e] > sp.printed_iso)) continue;
          for (int a = 0; a < 8; ++a) {
            const int ox = a & 1, oy = (a >> 1) & 1, oz = a >> 2;
            printed[size_t((int64_t(k + oz) * g.nny + (j + oy)) * g.nnx + (i + ox))] = 1;
          }
        }
    for (int64_t n = 0; n < g.nnodes; ++n)
      if (!printed[size_t(n)]) disp_out[3 * n] = disp_out[3 * n + 1] = disp_out[3 * n + 2] = 0.0;
  }
}

// A job that only solves: the analysis grid, its BCs and loads, the solve form
// and tolerance (tg_simp_compliance builds the same).
std::unique_ptr<tg_job> solve_only_job(const tg_grid* grid, const tg_simp_params* params,
                                       const tg_dirichlet_bc* bcs, int nbc,
                                       const tg_nodal_load* loads, int nloads, double tol,
                                       int max_it, const tg_solve_options* solve) {
  tg_simp_options o;
  std::memset(&o, 0, sizeof o);
  o.volume_fraction = 0.5;
  o.filter_radius = 1.5;
  o.move = 0.2;
  o.max_iterations = 1;
  o.cg_tolerance = tol > 0.0 ? tol : 1e-8;
  o.cg_max_iterations = max_it;
  if (solve) o.solve = *solve;
  auto jp = std::make_unique<tg_job>();
  job_init(jp.get(), grid, params, bcs, nbc, loads, nloads, &o);
  return jp;
}

// make_density_filter(grid, radius[, mask]) and one filter pass: the design set
// is the solid voxels, and with a mask the solid voxels whose entry is Active
// (simp.cpp:846-849).
void filter_call(const tg_grid* grid, const uint8_t* mask, double radius, int adjoint,
                 const double* x, double* out) {
  validate_grid(grid);
  if (!x || !out) raise(TG_EINVAL, "x and out must be non-null");
  CallStream cs;
  const Grid g = Grid::make(grid->nx, grid->ny, grid->nz, grid->spacing);
  std::vector<uint8_t> act(size_t(g.nv));
  for (int64_t e = 0; e < g.nv; ++e)
    act[size_t(e)] = (grid->tags == nullptr || grid->tags[e] != 0) && (!mask || mask[e] == 0);
  DBuf<uint8_t> dact;
  DBuf<double> dx, dout(size_t(g.nv));
  upload(dact, act.data(), act.size(), cs.s);
  upload(dx, x, size_t(g.nv), cs.s);
  FilterState fs;
  fs.init(g, radius, dact.p, cs.s);
  if (adjoint)
    fs.adj(g, dact.p, dx.p, dout.p, cs.s);
  else
    fs.fwd(g, dact.p, dx.p, dout.p, cs.s);
  TG_CUDA(cudaMemcpyAsync(out, dout.p, dout.bytes(), cudaMemcpyDeviceToHost, cs.s));
  TG_CUDA(cudaStreamSynchronize(cs.s));
}

// oc_update (simp.cpp:948-1025) when eff is null; oc_update_masked
// (simp.cpp:2662-2720) with the effective mask eff: the design set is the
// Active voxels, the filter is Active-only and frozen voxels keep their x.
void oc_call(const tg_grid* grid, const uint8_t* eff, double radius, const double* density,
             const double* dc, double volfrac, double move, double rho_min, double* x_new) {
  validate_grid(grid);
  if (!density || !dc || !x_new) raise(TG_EINVAL, "density, dc and x_new must be non-null");
  if (!(volfrac > 0.0 && volfrac <= 1.0))
    raise(TG_EINVAL, "oc_update: volume_fraction must be in (0, 1]");
  if (!(move > 0.0)) raise(TG_EINVAL, "oc_update: move must be > 0");
  if (!(rho_min > 0.0 && rho_min <= 1.0))
    raise(TG_EINVAL, "oc_update: density_min must be in (0, 1]");
  CallStream cs;
  const Grid g = Grid::make(grid->nx, grid->ny, grid->nz, grid->spacing);
  std::vector<uint8_t> act(size_t(g.nv));
  int64_t n_design = 0;
  for (int64_t e = 0; e < g.nv; ++e) {
    act[size_t(e)] = eff ? eff[e] == 0 : (grid->tags == nullptr || grid->tags[e] != 0);
    n_design += act[size_t(e)];
  }
  DBuf<uint8_t> dact;
  DBuf<double> dx, ddc, dxn(size_t(g.nv)), ones;
  upload(dact, act.data(), act.size(), cs.s);
  upload(dx, density, size_t(g.nv), cs.s);
  upload(ddc, dc, size_t(g.nv), cs.s);
  std::vector<double> o1(size_t(g.nv));
  for (int64_t e = 0; e < g.nv; ++e) o1[size_t(e)] = act[size_t(e)] ? 1.0 : 0.0;
  upload(ones, o1.data(), o1.size(), cs.s);
  FilterState fs;
  fs.init(g, radius, dact.p, cs.s);
  OcState oc;
  oc.init(g, cs.s);
  oc.n_solid = n_design;
  oc.carry = eff != nullptr;
  fs.adj(g, dact.p, ones.p, oc.dvf.p, cs.s);
  oc_update_device(oc, fs, g, dact.p, act, dx.p, ddc.p, volfrac, move, rho_min, dxn.p, cs.s);
  TG_CUDA(cudaMemcpyAsync(x_new, dxn.p, dxn.bytes(), cudaMemcpyDeviceToHost, cs.s));
  TG_CUDA(cudaStreamSynchronize(cs.s));
}
}  // namespace
}  // namespace tg

// ================================================================= C ABI
extern "C" {

const char* tg_last_error(void) { return tg::g_err.c_str(); }

int tg_set_device(int32_t device) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n) {
    tg::g_err = "tg_set_device: no such CUDA device";
    return TG_EINVAL;
  }
  tg::g_device = device;
  return TG_OK;
}

const char* tg_version(void) { return "topopt_gb300 0.1 (sm_103a)"; }

int tg_set_sync_mode(int32_t mode) {
  static const unsigned kFlags[4] = {cudaDeviceScheduleAuto, cudaDeviceScheduleSpin,
                                     cudaDeviceScheduleYield, cudaDeviceScheduleBlockingSync};
  if (mode < 0 || mode > 3) {
    tg::g_err = "tg_set_sync_mode: mode must be 0..3";
    return TG_EINVAL;
  }
  return guarded([&] { TG_CUDA(cudaSetDeviceFlags(kFlags[mode])); });
}

int tg_hex8_stiffness(double E, double nu, double h, double* ke) {
  try {
    if (!ke) raise(TG_EINVAL, "ke is null");
    if (!(E > 0.0)) raise(TG_EINVAL, "hex8_stiffness: youngs_modulus must be > 0");
    if (!(h > 0.0)) raise(TG_EINVAL, "hex8_stiffness: element_size must be > 0");
    if (!(nu > -1.0 && nu < 0.5)) raise(TG_EINVAL, "hex8_stiffness: poisson must be in (-1, 0.5)");
    hex8_ke(E, nu, h, ke);
    return TG_OK;
  } catch (const Error& e) {
    tg::g_err = e.what();
    return e.code;
  }
}

int tg_matfree_apply(const tg_grid* grid, double E, double nu, const double* youngs,
                     int32_t precision, const double* u, double* y) {
  return guarded([&] {
    validate_grid(grid);
    if (!u || !y) raise(TG_EINVAL, "u and y must be non-null");
    if (!youngs && !(E > 0.0)) raise(TG_EINVAL, "hex8_stiffness: youngs_modulus must be > 0");
    if (!(nu > -1.0 && nu < 0.5)) raise(TG_EINVAL, "hex8_stiffness: poisson must be in (-1, 0.5)");
    CallStream cs;
    const Grid g = Grid::make(grid->nx, grid->ny, grid->nz, grid->spacing);
    std::vector<double> f(size_t(g.nv), 0.0);
    for (int64_t e = 0; e < g.nv; ++e) {
      const bool sol = grid->tags == nullptr || grid->tags[e] != 0;
      if (!sol) continue;
      f[size_t(e)] = youngs ? youngs[e] : E;
      if (youngs && !(youngs[e] > 0.0))
        raise(TG_EINVAL,
              "fea_matfree_apply: per-voxel Young's modulus must be > 0 on a solid voxel");
    }
    ModalConsts mc = ModalConsts::make(nu, g.h);
    DBuf<double> df, du, dy;
    upload(df, f.data(), f.size(), cs.s);
    upload(du, u, size_t(g.ndof), cs.s);
    dy.alloc(size_t(g.ndof));
    if (precision == TG_PREC_MIXED) {
      DBuf<float> ff(size_t(g.nv)), fu(size_t(g.ndof)), fy(size_t(g.ndof));
      launch_copy_d2f(ff.p, df.p, g.nv, cs.s);
      launch_copy_d2f(fu.p, du.p, g.ndof, cs.s);
      launch_fine_op<float>(kApply, g, mc, ff.p, nullptr, fu.p, nullptr, nullptr, 0.0f, fy.p,
                            nullptr, nullptr, cs.s);
      std::vector<float> hy(size_t(g.ndof));
      TG_CUDA(cudaMemcpyAsync(hy.data(), fy.p, fy.bytes(), cudaMemcpyDeviceToHost, cs.s));
      TG_CUDA(cudaStreamSynchronize(cs.s));
      for (int64_t d = 0; d < g.ndof; ++d) y[d] = double(hy[size_t(d)]);
      return;
    }
    if (precision == TG_APPLY_DF) {
      // y = -(0 - A u): the double-float residual kernel with b = 0.
      DBuf<double> zero(size_t(g.ndof));
      TG_CUDA(cudaMemsetAsync(zero.p, 0, zero.bytes(), cs.s));
      launch_fine_residual_df(g, mc, df.p, nullptr, du.p, zero.p, dy.p, cs.s);
      TG_CUDA(cudaMemcpyAsync(y, dy.p, dy.bytes(), cudaMemcpyDeviceToHost, cs.s));
      TG_CUDA(cudaStreamSynchronize(cs.s));
      for (int64_t d = 0; d < g.ndof; ++d) y[d] = -y[d];
      return;
    }
    launch_fine_op<double>(kApply, g, mc, df.p, nullptr, du.p, nullptr, nullptr, 0.0, dy.p,
                           nullptr, nullptr, cs.s);
    TG_CUDA(cudaMemcpyAsync(y, dy.p, dy.bytes(), cudaMemcpyDeviceToHost, cs.s));
    TG_CUDA(cudaStreamSynchronize(cs.s));
  });
}

int tg_build_reduced(const tg_grid* grid, const double* youngs, double nu,
                     const tg_dirichlet_bc* bcs, int32_t nbc, const tg_nodal_load* loads,
                     int32_t nloads, uint8_t* kept, double* rhs, double* invdiag,
                     int32_t* ng_out) {
  return guarded([&] {
    validate_grid(grid);
    CallStream cs;
    FineProblem fp;
    fp.build(*grid, nu, bcs, nbc, loads, nloads, nullptr, cs.s);
    const Grid& g = fp.g;
    std::vector<double> f(size_t(g.nv), 0.0);
    for (int64_t e = 0; e < g.nv; ++e)
      if (fp.elem_h[size_t(e)]) {
        f[size_t(e)] = youngs ? youngs[e] : 1.0;
        if (!(f[size_t(e)] > 0.0))
          raise(TG_EINVAL, "per-voxel Young's modulus must be > 0 on a solid voxel");
      }
    DBuf<double> dE;
    upload(dE, f.data(), f.size(), cs.s);
    tg_solve_options so;
    std::memset(&so, 0, sizeof so);
    so.solver = TG_SOLVER_JACOBI_CG;
    Solver sv(fp, so, cs.s);
    sv.set_modulus(dE.p);
    std::vector<double> tmp(size_t(g.ndof));
    if (rhs) {
      TG_CUDA(cudaMemcpyAsync(rhs, sv.rhs(), size_t(g.ndof) * sizeof(double),
                              cudaMemcpyDeviceToHost, cs.s));
    }
    TG_CUDA(cudaStreamSynchronize(cs.s));
    if (kept) std::memcpy(kept, fp.kept_h.data(), size_t(g.ndof));
    if (invdiag) {
      DBuf<double> inv(size_t(g.ndof));
      launch_fine_invdiag(g, fp.mc.kdiag, dE.p, fp.kept.p, inv.p, cs.s);
      TG_CUDA(cudaMemcpyAsync(invdiag, inv.p, inv.bytes(), cudaMemcpyDeviceToHost, cs.s));
      TG_CUDA(cudaStreamSynchronize(cs.s));
    }
    if (ng_out) *ng_out = int32_t(fp.ng);
  });
}

int tg_solve(const tg_grid* grid, const double* youngs, double nu, const tg_dirichlet_bc* bcs,
             int32_t nbc, const tg_nodal_load* loads, int32_t nloads, double tol, int32_t max_it,
             const tg_solve_options* options, const uint8_t* active_mask, const double* guess,
             double* u_out, tg_cg_info* info) {
  SolverStats st;
  FineProblem fp;
  double t_build = 0.0;
  const double t0 = now_ms();
  const int rc = guarded([&] {
    validate_grid(grid);
    if (!youngs || !u_out) raise(TG_EINVAL, "youngs_per_voxel and u_out must be non-null");
    const tg_solve_options so = default_solve(options);
    CallStream cs;
    fp.build(*grid, nu, bcs, nbc, loads, nloads, active_mask, cs.s);
    const Grid& g = fp.g;
    std::vector<double> f(size_t(g.nv), 0.0);
    for (int64_t e = 0; e < g.nv; ++e)
      if (fp.elem_h[size_t(e)]) {
        f[size_t(e)] = youngs[e];
        if (!(youngs[e] > 0.0))
          raise(TG_EINVAL,
                "fea_solve_mgcg_matfree: per-voxel Young's modulus must be > 0 on a solid voxel");
      }
    DBuf<double> dE, du, dg;
    upload(dE, f.data(), f.size(), cs.s);
    du.alloc(size_t(g.ndof));
    if (guess) upload(dg, guess, size_t(g.ndof), cs.s);
    Solver sv(fp, so, cs.s);
    const double tb = now_ms();
    sv.set_modulus(dE.p);
    TG_CUDA(cudaStreamSynchronize(cs.s));
    st = sv.solve(tol, max_it, guess ? dg.p : nullptr, du.p);
    st.t_mg_build_ms = now_ms() - tb - st.t_solve_ms;
    t_build = tb - t0;
    if (!st.converged) {
      Error e(TG_ENONCONV,
              "fea_solve_mgcg_matfree: CG did not reach the requested tolerance within "
              "max_iterations");
      throw e;
    }
    TG_CUDA(cudaMemcpyAsync(u_out, du.p, du.bytes(), cudaMemcpyDeviceToHost, cs.s));
    TG_CUDA(cudaStreamSynchronize(cs.s));
  });
  fill_info(info, st, fp, t_build, now_ms() - t0);
  return rc;
}

int tg_simp_compliance(const tg_grid* grid, const tg_simp_params* params, const double* density,
                       const tg_dirichlet_bc* bcs, int32_t nbc, const tg_nodal_load* loads,
                       int32_t nloads, double tol, int32_t max_it,
                       const tg_solve_options* options, double* u_out, double* dc_out,
                       double* compliance_out, tg_cg_info* info) {
  SolverStats st;
  std::unique_ptr<tg_job> jp;
  const double t0 = now_ms();
  const int rc = guarded([&] {
    validate_grid(grid);
    validate_params(params);
    if (!density) raise(TG_EINVAL, "density is null");
    jp = solve_only_job(grid, params, bcs, nbc, loads, nloads, tol, max_it, options);
    tg_job* j = jp.get();
    const tg_simp_options& o = j->opt;
    const Grid& g = j->fp.g;
    TG_CUDA(cudaMemcpyAsync(j->xphys.p, density, j->xphys.bytes(), cudaMemcpyHostToDevice, j->s));
    j->xphys_valid = true;
    st = job_solve(j, o.cg_tolerance, max_it);
    if (!st.converged) raise(TG_ENONCONV, "simp_compliance: CG did not reach the requested tolerance");
    const double c = job_sensitivity(j);
    if (compliance_out) *compliance_out = c;
    if (u_out)
      TG_CUDA(cudaMemcpyAsync(u_out, j->u.p, j->u.bytes(), cudaMemcpyDeviceToHost, j->s));
    if (dc_out)
      TG_CUDA(cudaMemcpyAsync(dc_out, j->dc.p, size_t(g.nv) * sizeof(double),
                              cudaMemcpyDeviceToHost, j->s));
    TG_CUDA(cudaStreamSynchronize(j->s));
  });
  if (jp) fill_info(info, st, jp->fp, 0.0, now_ms() - t0);
  return rc;
}

int tg_filter(const tg_grid* grid, double radius, int32_t adjoint, const double* x, double* out) {
  return guarded([&] { filter_call(grid, nullptr, radius, adjoint, x, out); });
}

int tg_filter_masked(const tg_grid* grid, const uint8_t* mask, double radius, int32_t adjoint,
                     const double* x, double* out) {
  return guarded([&] {
    validate_grid(grid);
    if (!mask) raise(TG_EINVAL, "make_density_filter: mask size != voxel_count");
    filter_call(grid, mask, radius, adjoint, x, out);
  });
}

int tg_oc_update(const tg_grid* grid, double radius, const double* density, const double* dc,
                 double volfrac, double move, double rho_min, double* x_new) {
  return guarded(
      [&] { oc_call(grid, nullptr, radius, density, dc, volfrac, move, rho_min, x_new); });
}

int tg_oc_update_masked(const tg_grid* grid, const uint8_t* mask, double radius,
                        const double* density, const double* dc, double volfrac, double move,
                        double rho_min, double* x_new) {
  return guarded([&] {
    validate_grid(grid);
    const std::vector<uint8_t> eff = effective_mask(grid, mask, "oc_update_masked");
    oc_call(grid, eff.data(), radius, density, dc, volfrac, move, rho_min, x_new);
  });
}

int tg_heaviside_project(int64_t n, const double* rho_tilde, double beta, double eta,
                         double* value, double* derivative) {
  return guarded([&] {
    // validate_projection_args (simp.cpp:49-55).
    if (!(beta > 0.0) || !std::isfinite(beta))
      raise(TG_EINVAL, "heaviside_project: beta must be finite and > 0");
    if (!(eta > 0.0 && eta < 1.0)) raise(TG_EINVAL, "heaviside_project: eta must be in (0, 1)");
    if (n < 0 || (n > 0 && !rho_tilde)) raise(TG_EINVAL, "rho_tilde must hold n values");
    if (n == 0 || (!value && !derivative)) return;
    CallStream cs;
    DBuf<double> drt, dv, dd;
    upload(drt, rho_tilde, size_t(n), cs.s);
    if (value) dv.alloc(size_t(n));
    if (derivative) dd.alloc(size_t(n));
    launch_project(drt.p, nullptr, n, beta, eta, dv.p, dd.p, cs.s);
    if (value)
      TG_CUDA(cudaMemcpyAsync(value, dv.p, dv.bytes(), cudaMemcpyDeviceToHost, cs.s));
    if (derivative)
      TG_CUDA(cudaMemcpyAsync(derivative, dd.p, dd.bytes(), cudaMemcpyDeviceToHost, cs.s));
    TG_CUDA(cudaStreamSynchronize(cs.s));
  });
}

int32_t tg_heaviside_continuation_schedule(tg_projection_stage* out, int32_t cap) {
  static const tg_projection_stage kSchedule[6] = {
      {1.0, 0.2, 50}, {2.0, 0.2, 50}, {4.0, 0.2, 50}, {8.0, 0.2, 50}, {16.0, 0.1, 50},
      {32.0, 0.05, 50}};
  for (int i = 0; out && i < cap && i < 6; ++i) out[i] = kSchedule[i];
  return 6;
}

int tg_oc_update_projected(const tg_grid* grid, double radius, const double* density,
                           const double* xtilde, const double* dcompliance, double beta,
                           double eta, double volume_fraction, double move, double density_min,
                           double* x_new) {
  return guarded([&] {
    validate_grid(grid);
    if (!density || !xtilde || !dcompliance || !x_new)
      raise(TG_EINVAL, "density, xtilde, dcompliance and x_new must be non-null");
    if (!(beta > 0.0) || !std::isfinite(beta))
      raise(TG_EINVAL, "heaviside_project: beta must be finite and > 0");
    if (!(eta > 0.0 && eta < 1.0)) raise(TG_EINVAL, "heaviside_project: eta must be in (0, 1)");
    CallStream cs;
    const Grid g = Grid::make(grid->nx, grid->ny, grid->nz, grid->spacing);
    std::vector<uint8_t> act(size_t(g.nv));
    int64_t n_design = 0;
    for (int64_t e = 0; e < g.nv; ++e) {
      act[size_t(e)] = grid->tags == nullptr || grid->tags[e] != 0;
      n_design += act[size_t(e)];
    }
    DBuf<uint8_t> dact;
    DBuf<double> dx, dxt, ddc, dxn(size_t(g.nv));
    upload(dact, act.data(), act.size(), cs.s);
    upload(dx, density, size_t(g.nv), cs.s);
    upload(dxt, xtilde, size_t(g.nv), cs.s);
    upload(ddc, dcompliance, size_t(g.nv), cs.s);
    FilterState fs;
    fs.init(g, radius, dact.p, cs.s);
    OcState oc;
    oc.init(g, cs.s);
    oc.n_solid = n_design;
    oc_update_projected_device(oc, fs, g, dact.p, dx.p, dxt.p, ddc.p, beta, eta, volume_fraction,
                               move, density_min, dxn.p, cs.s);
    TG_CUDA(cudaMemcpyAsync(x_new, dxn.p, dxn.bytes(), cudaMemcpyDeviceToHost, cs.s));
    TG_CUDA(cudaStreamSynchronize(cs.s));
  });
}

int tg_effective_design_mask(const tg_grid* grid, const uint8_t* mask, uint8_t* eff_out) {
  return guarded([&] {
    validate_grid(grid);
    if (!eff_out) raise(TG_EINVAL, "eff_out is null");
    const std::vector<uint8_t> eff = effective_mask(grid, mask, "effective_design_mask");
    std::memcpy(eff_out, eff.data(), eff.size());
  });
}

int32_t tg_active_domain_auto_band(double filter_radius) {
  if (!std::isfinite(filter_radius) || filter_radius <= 0.0) return 1;
  const int k = static_cast<int>(std::ceil(filter_radius)) + 1;
  return k < 1 ? 1 : k;
}

int tg_active_domain_mask(const tg_grid* grid, const double* density, double density_min,
                          int32_t band, uint8_t* mask_out, int64_t* active_count) {
  return guarded([&] {
    validate_grid(grid);
    if (!density || !mask_out) raise(TG_EINVAL, "density and mask_out must be non-null");
    CallStream cs;
    const int64_t nv = int64_t(grid->nx) * grid->ny * grid->nz;
    DBuf<uint8_t> tags, out{static_cast<size_t>(nv)}, tmp{static_cast<size_t>(nv)};
    DBuf<double> rho;
    DBuf<unsigned long long> count(1);
    if (grid->tags) upload(tags, grid->tags, size_t(nv), cs.s);
    upload(rho, density, size_t(nv), cs.s);
    launch_active_domain_mask(grid->nx, grid->ny, grid->nz, tags.p, rho.p, density_min, band,
                              out.p, tmp.p, count.p, cs.s);
    unsigned long long n = 0;
    TG_CUDA(cudaMemcpyAsync(mask_out, out.p, size_t(nv), cudaMemcpyDeviceToHost, cs.s));
    TG_CUDA(cudaMemcpyAsync(&n, count.p, sizeof n, cudaMemcpyDeviceToHost, cs.s));
    TG_CUDA(cudaStreamSynchronize(cs.s));
    if (active_count) *active_count = int64_t(n);
  });
}

int tg_active_domain_escape_count(const tg_grid* grid, const double* density,
                                  const uint8_t* prev_mask, double density_min,
                                  int64_t* escapes) {
  return guarded([&] {
    validate_grid(grid);
    if (!density || !escapes) raise(TG_EINVAL, "density and escapes must be non-null");
    *escapes = 0;
    if (!prev_mask) return;  // the first armed iteration: no band to overrun
    CallStream cs;
    const int64_t nv = int64_t(grid->nx) * grid->ny * grid->nz;
    DBuf<uint8_t> tags, prev;
    DBuf<double> rho;
    DBuf<unsigned long long> count(1);
    if (grid->tags) upload(tags, grid->tags, size_t(nv), cs.s);
    upload(prev, prev_mask, size_t(nv), cs.s);
    upload(rho, density, size_t(nv), cs.s);
    launch_active_domain_escape(tags.p, rho.p, prev.p, density_min, nv, count.p, cs.s);
    unsigned long long n = 0;
    TG_CUDA(cudaMemcpyAsync(&n, count.p, sizeof n, cudaMemcpyDeviceToHost, cs.s));
    TG_CUDA(cudaStreamSynchronize(cs.s));
    *escapes = int64_t(n);
  });
}

int tg_job_create(const tg_grid* grid, const tg_simp_params* params, const tg_dirichlet_bc* bcs,
                  int32_t nbc, const tg_nodal_load* loads, int32_t nloads,
                  const tg_simp_options* options, tg_job** job_out) {
  return guarded([&] {
    if (!job_out) raise(TG_EINVAL, "job_out is null");
    auto j = std::make_unique<tg_job>();
    job_init(j.get(), grid, params, bcs, nbc, loads, nloads, options);
    *job_out = j.release();
  });
}

int tg_job_create_masked(const tg_grid* grid, const tg_simp_params* params,
                         const tg_dirichlet_bc* bcs, int32_t nbc, const tg_nodal_load* loads,
                         int32_t nloads, const tg_simp_options* options, const uint8_t* mask,
                         tg_job** job_out) {
  return guarded([&] {
    if (!job_out) raise(TG_EINVAL, "job_out is null");
    validate_grid(grid);
    if (!mask) raise(TG_EINVAL, "simp_optimize: mask size != voxel_count");
    auto j = std::make_unique<tg_job>();
    job_init(j.get(), grid, params, bcs, nbc, loads, nloads, options, mask);
    *job_out = j.release();
  });
}

int tg_job_step(tg_job* job, tg_simp_iteration* row) {
  tg_simp_iteration r;
  std::memset(&r, 0, sizeof r);
  const int rc = guarded([&] {
    if (!job) raise(TG_EINVAL, "job is null");
    job_step(job, &r);
  });
  if (row) *row = r;
  return rc;
}

int tg_job_set_stage(tg_job* job, int32_t stage) {
  return guarded([&] {
    if (!job) raise(TG_EINVAL, "job is null");
    if (stage < 0 || stage >= std::max<int>(1, int(job->stages.size())))
      raise(TG_EINVAL, "tg_job_set_stage: stage outside the projection plan");
    if (job->stage != stage) {
      job->stage = stage;
      job->xphys_valid = false;
    }
  });
}

int tg_job_read(tg_job* job, double* design_out, double* phys_out) {
  return guarded([&] {
    if (!job) raise(TG_EINVAL, "job is null");
    const Grid& g = job->fp.g;
    if (!job->xphys_valid) job_filter_x(job);
    if (design_out)
      TG_CUDA(cudaMemcpyAsync(design_out, job->x.p, size_t(g.nv) * sizeof(double),
                              cudaMemcpyDeviceToHost, job->s));
    if (phys_out)
      TG_CUDA(cudaMemcpyAsync(phys_out, job->xphys.p, size_t(g.nv) * sizeof(double),
                              cudaMemcpyDeviceToHost, job->s));
    TG_CUDA(cudaStreamSynchronize(job->s));
  });
}

int tg_job_read_displacement(tg_job* job, double* u_out) {
  return guarded([&] {
    if (!job || !u_out) raise(TG_EINVAL, "job and u_out must be non-null");
    TG_CUDA(cudaMemcpyAsync(u_out, job->u.p, job->u.bytes(), cudaMemcpyDeviceToHost, job->s));
    TG_CUDA(cudaStreamSynchronize(job->s));
  });
}

int tg_job_write_design(tg_job* job, const double* design) {
  return guarded([&] {
    if (!job || !design) raise(TG_EINVAL, "job and design must be non-null");
    TG_CUDA(cudaMemcpyAsync(job->x.p, design, job->x.bytes(), cudaMemcpyHostToDevice, job->s));
    job->xphys_valid = false;
    TG_CUDA(cudaStreamSynchronize(job->s));
  });
}

void* tg_host_alloc(int64_t bytes) {
  if (bytes <= 0) return nullptr;
  void* p = nullptr;
  if (cudaHostAlloc(&p, size_t(bytes), cudaHostAllocDefault) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return p;
}

int tg_host_free(void* ptr) {
  if (ptr == nullptr) return TG_OK;  // like free(NULL): no device needed
  return guarded([&] { TG_CUDA(cudaFreeHost(ptr)); });
}

int64_t tg_job_device_bytes(const tg_job* job) { return job ? int64_t(job->bytes()) : 0; }

int64_t tg_job_estimate_bytes(const tg_grid* grid, const tg_simp_options* options) {
  if (!grid || grid->nx < 1 || grid->ny < 1 || grid->nz < 1) return -1;
  const double nv = double(grid->nx) * grid->ny * grid->nz;
  const double ndof = 3.0 * (grid->nx + 1.0) * (grid->ny + 1.0) * (grid->nz + 1.0);
  const bool mixed = options && options->solve.precision == TG_PREC_MIXED;
  // Fine: 9 FP64 DOF vectors + kept/f/up; ~12 voxel arrays.  Hierarchy: the
  // level-1 element matrices (576 doubles per 8 voxels) and stencils (126
  // doubles per node / 8), a geometric series over the coarser levels.
  double b = ndof * (9 * 8 + 1 + 16) + ndof / 3.0 + nv * (12 * 8 + 2);
  b += (nv / 8.0) * 576 * 8 * 8.0 / 7.0 + (ndof / 3.0 / 8.0) * 126 * 8 * 8.0 / 7.0;
  if (mixed) b += ndof * 8 * 4 + (ndof / 3.0 / 8.0) * 126 * 4 * 8.0 / 7.0 + nv * 4;
  if (options && options->projection_stages > 0)  // xtilde and the candidate fields
    b += nv * 8.0 * (1 + projected_candidates(int64_t(nv)));
  if (options && options->updater == TG_UPDATER_MMA) b += nv * 8.0 * 10;  // MMA fields
  if (options && options->active_domain_band != 0) {
    // The restricted system: its own reduced problem, solver vectors and
    // hierarchy (at most the full system's), and three byte masks.
    double r = ndof * (9 * 8 + 1 + 16) + ndof / 3.0 + nv * 4;
    r += (nv / 8.0) * 576 * 8 * 8.0 / 7.0 + (ndof / 3.0 / 8.0) * 126 * 8 * 8.0 / 7.0;
    if (mixed) r += ndof * 8 * 4 + (ndof / 3.0 / 8.0) * 126 * 4 * 8.0 / 7.0 + nv * 4;
    b += r;
  }
  return int64_t(b * 1.05) + (64 << 20);
}

void tg_job_destroy(tg_job* job) { delete job; }

int tg_job_time_operator(tg_job* job, int32_t precision, int32_t reps, double* avg_ms) {
  return guarded([&] {
    if (!job || !avg_ms || reps < 1) raise(TG_EINVAL, "job, avg_ms and reps >= 1 required");
    AllocScope scope(job->s);
    if (!job->xphys_valid) job_filter_x(job);
    const Grid& g = job->fp.g;
    const tg_simp_params& p = job->params;
    launch_modulus(job->xphys.p, job->fp.elem.p, g.nv, p.youngs_modulus, p.penalty,
                   p.density_min, p.material_law, p.e_min, job->E.p, job->s);
    job->solver->set_modulus(job->E.p);
    *avg_ms = job->solver->time_operator(precision == TG_PREC_MIXED       ? 1
                                         : precision == TG_APPLY_DF         ? 2
                                         : precision == TG_APPLY_L1_STENCIL ? 3
                                         : precision == TG_APPLY_L1_TC      ? 4
                                                                            : 0,
                                         reps);
  });
}

int tg_job_check_level1(tg_job* job, double* rel_diff) {
  return guarded([&] {
    if (!job || !rel_diff) raise(TG_EINVAL, "job and rel_diff required");
    AllocScope scope(job->s);
    if (!job->xphys_valid) job_filter_x(job);
    const tg_simp_params& p = job->params;
    launch_modulus(job->xphys.p, job->fp.elem.p, job->fp.g.nv, p.youngs_modulus, p.penalty,
                   p.density_min, p.material_law, p.e_min, job->E.p, job->s);
    job->solver->set_modulus(job->E.p);
    *rel_diff = job->solver->check_level1();
  });
}

int64_t tg_kernel_launches(void) { return tg::g_launches.load(); }

int tg_set_level1_tc(int32_t on) {
  return guarded([&] { set_level1_tc(on != 0); });
}

int tg_set_level1_galerkin_fast(int32_t on) {
  return guarded([&] { set_level1_galerkin_fast(on != 0); });
}

int tg_set_coarse_fused(int32_t on) {
  return guarded([&] { set_coarse_fused(on != 0); });
}

int tg_set_fp32_schedule(int32_t kind, int32_t shape, int32_t kz) {
  return guarded([&] {
    if (kind < 0) {
      set_fine_schedule_override(nullptr);
      return;
    }
    FineSchedule s;
    s.kind = kind;
    s.shape = shape;
    s.kz = kz;
    if (!fine_schedule_valid(s)) raise(TG_EINVAL, "tg_set_fp32_schedule: no such schedule");
    set_fine_schedule_override(&s);
  });
}

int tg_fp32_schedule(int32_t nx, int32_t ny, int32_t nz, int32_t* kind, int32_t* shape,
                     int32_t* kz) {
  return guarded([&] {
    if (nx < 1 || ny < 1 || nz < 1) raise(TG_EINVAL, "grid dimensions must be >= 1");
    const FineSchedule s = fine_schedule_for(Grid::make(nx, ny, nz, 1.0));
    if (kind) *kind = s.kind;
    if (shape) *shape = s.shape;
    if (kz) *kz = s.kz;
  });
}

int tg_device_fma_peaks(double* fp64_tflops, double* fp32_tflops) {
  return guarded([&] {
    if (fp64_tflops) *fp64_tflops = fma_probe_tflops(true);
    if (fp32_tflops) *fp32_tflops = fma_probe_tflops(false);
  });
}

static int simp_optimize_impl(const tg_grid* grid, const tg_simp_params* params,
                              const tg_dirichlet_bc* bcs, int32_t nbc, const tg_nodal_load* loads,
                              int32_t nloads, const tg_simp_options* options,
                              const uint8_t* mask, tg_progress_fn progress, void* progress_ctx,
                              const volatile int32_t* cancel, tg_simp_iteration* history,
                              double* design_out, double* phys_out, tg_simp_result* result) {
  tg_simp_result res;
  std::memset(&res, 0, sizeof res);
  const int rc = guarded([&] {
    auto jp = std::make_unique<tg_job>();
    job_init(jp.get(), grid, params, bcs, nbc, loads, nloads, options, mask);
    tg_job* j = jp.get();
    const tg_simp_options& o = j->opt;
    // The stage plan (simp.cpp:2158-2507): one unprojected stage of
    // max_iterations, or the projection stages in order, each ended early by
    // change < change_tol; the run is converged iff its last stage was.
    const int nst = j->projecting() ? int(j->stages.size()) : 1;
    bool stop = false;
    int nrow = 0;
    for (int si = 0; si < nst && !stop; ++si) {
      if (j->projecting() && j->stage != si) {
        j->stage = si;
        j->xphys_valid = false;  // xPhys is projected at the new stage's beta
      }
      const int iters = j->projecting() ? j->stages[size_t(si)].iterations : o.max_iterations;
      bool stage_conv = false;
      for (int it = 0; it < iters; ++it) {
        if (cancel && *cancel) {
          res.cancelled = 1;
          stop = true;
          break;
        }
        tg_simp_iteration row;
        try {
          job_step(j, &row);
        } catch (const Error& e) {
          if (e.code != TG_ENONCONV) throw;
          res.non_convergent = 1;  // simp.cpp:2254-2266: ends the run, no throw
          stop = true;
          break;
        }
        if (history) history[nrow] = row;
        if (nrow == 0) res.initial_compliance = row.compliance;
        ++nrow;
        res.iterations = j->iteration;
        if (progress) progress(progress_ctx, row.iteration, row.compliance, row.change);
        if (rung_infeasible(j->hist_c, j->hist_cg)) {
          res.infeasible = 1;
          stop = true;
          break;
        }
        // stage_should_stop (simp.cpp:1219-1233): MMA on the objective plateau.
        const bool stop_here = (j->mma && o.mma_plateau_window > 0)
                                   ? mma_objective_plateau(j->hist_c, o)
                                   : row.change < o.change_tol;
        if (stop_here) {
          stage_conv = true;
          break;
        }
      }
      res.converged = stage_conv ? 1 : 0;
    }
    const Grid& g = j->fp.g;
    // physical_density = filter(design), projected at the LAST stage's beta
    // (simp.cpp:2514-2517), whatever stage the loop stopped in.
    if (j->projecting()) j->stage = nst - 1;
    job_filter_x(j);
    if (res.infeasible || res.non_convergent || res.cancelled) {
      res.compliance = j->hist_c.empty() ? 0.0 : j->hist_c.back();
    } else {
      // The certification solve at the tight tolerance (simp.cpp:2566-2570).
      const SolverStats st = job_solve(j, o.cg_tolerance, o.cg_max_iterations);
      if (!st.converged) {
        res.non_convergent = 1;
        res.converged = 0;
        res.compliance = j->hist_c.empty() ? 0.0 : j->hist_c.back();
      } else {
        res.compliance = job_sensitivity(j);
      }
    }
    bool exact = false;
    const double vol = exact_volume(j->oc, g, j->solid.p, j->xphys.p, &exact, j->s);
    res.volume_fraction = j->n_solid > 0 ? vol / double(j->n_solid) : 0.0;
    // finalize_active_domain (simp.cpp:1981-1988), after the full-domain
    // certification solve.
    const tg_job::ActiveDomain& ad = j->ad;
    res.active_domain_band = ad.band;
    res.active_domain_latched = ad.latched ? 1 : 0;
    res.active_domain_latch_iteration = ad.latch_iteration;
    res.active_domain_escape_count = ad.escape_count;
    res.active_fraction_mean =
        ad.fraction_count > 0 ? ad.fraction_sum / double(ad.fraction_count) : 1.0;
    std::snprintf(res.active_domain_latch_reason, sizeof res.active_domain_latch_reason, "%s",
                  ad.reason.c_str());
    if (design_out)
      TG_CUDA(cudaMemcpyAsync(design_out, j->x.p, size_t(g.nv) * sizeof(double),
                              cudaMemcpyDeviceToHost, j->s));
    if (phys_out)
      TG_CUDA(cudaMemcpyAsync(phys_out, j->xphys.p, size_t(g.nv) * sizeof(double),
                              cudaMemcpyDeviceToHost, j->s));
    TG_CUDA(cudaStreamSynchronize(j->s));
  });
  if (result) *result = res;
  return rc;
}

int tg_simp_optimize(const tg_grid* grid, const tg_simp_params* params,
                     const tg_dirichlet_bc* bcs, int32_t nbc, const tg_nodal_load* loads,
                     int32_t nloads, const tg_simp_options* options, tg_progress_fn progress,
                     void* progress_ctx, const volatile int32_t* cancel,
                     tg_simp_iteration* history, double* design_out, double* phys_out,
                     tg_simp_result* result) {
  return simp_optimize_impl(grid, params, bcs, nbc, loads, nloads, options, nullptr, progress,
                            progress_ctx, cancel, history, design_out, phys_out, result);
}

int tg_simp_optimize_masked(const tg_grid* grid, const tg_simp_params* params,
                            const tg_dirichlet_bc* bcs, int32_t nbc, const tg_nodal_load* loads,
                            int32_t nloads, const tg_simp_options* options, const uint8_t* mask,
                            tg_progress_fn progress, void* progress_ctx,
                            const volatile int32_t* cancel, tg_simp_iteration* history,
                            double* design_out, double* phys_out, tg_simp_result* result) {
  if (!mask) {
    tg::set_last_error("simp_optimize: mask size != voxel_count");
    if (result) std::memset(result, 0, sizeof *result);
    return TG_EINVAL;
  }
  return simp_optimize_impl(grid, params, bcs, nbc, loads, nloads, options, mask, progress,
                            progress_ctx, cancel, history, design_out, phys_out, result);
}

int tg_element_stress(const tg_grid* grid, double youngs_modulus, double poisson,
                      const double* u, const double* density, double iso, double* sigma_out,
                      double* von_mises_out) {
  return guarded([&] {
    validate_grid(grid);
    if (!u) raise(TG_EINVAL, "u is null");
    if (!(youngs_modulus > 0.0)) raise(TG_EINVAL, "hex8_stress: youngs_modulus must be > 0");
    if (!(grid->spacing > 0.0)) raise(TG_EINVAL, "hex8_stress: element_size must be > 0");
    if (!(poisson > -1.0 && poisson < 0.5))
      raise(TG_EINVAL, "hex8_stress: poisson must be in (-1, 0.5)");
    CallStream cs;
    const Grid g = Grid::make(grid->nx, grid->ny, grid->nz, grid->spacing);
    std::vector<uint8_t> solid(size_t(g.nv));
    for (int64_t e = 0; e < g.nv; ++e) solid[size_t(e)] = grid->tags == nullptr || grid->tags[e];
    DBuf<uint8_t> dsolid;
    DBuf<double> du, drho, dvm, dsig;
    upload(dsolid, solid.data(), solid.size(), cs.s);
    upload(du, u, size_t(g.ndof), cs.s);
    if (density) upload(drho, density, size_t(g.nv), cs.s);
    if (von_mises_out) dvm.alloc(size_t(g.nv));
    if (sigma_out) dsig.alloc(size_t(6 * g.nv));
    const double zdir[3] = {0.0, 0.0, 1.0};
    launch_element_stress(g, dsolid.p, drho.p, du.p, youngs_modulus, poisson, g.h, zdir, iso,
                          dvm.p, dsig.p, nullptr, cs.s);
    if (von_mises_out)
      TG_CUDA(cudaMemcpyAsync(von_mises_out, dvm.p, dvm.bytes(), cudaMemcpyDeviceToHost, cs.s));
    if (sigma_out)
      TG_CUDA(cudaMemcpyAsync(sigma_out, dsig.p, dsig.bytes(), cudaMemcpyDeviceToHost, cs.s));
    TG_CUDA(cudaStreamSynchronize(cs.s));
  });
}

int tg_load_path_connected(const tg_grid* grid, const double* density, double iso,
                           int32_t* connected) {
  return guarded([&] {
    validate_grid(grid);
    if (!density || !connected) raise(TG_EINVAL, "density and connected must be non-null");
    const Grid g = Grid::make(grid->nx, grid->ny, grid->nz, grid->spacing);
    *connected = load_path_host(g, grid->tags, density, iso) ? 1 : 0;
  }, /*device=*/false);
}

int tg_analyze_fixed_design(const tg_grid* grid, const tg_simp_params* params,
                            const double* density, const tg_dirichlet_bc* bcs, int32_t nbc,
                            const tg_nodal_load* loads, int32_t nloads,
                            const tg_strength_spec* strength, double cg_tolerance,
                            int32_t cg_max_iterations, const tg_solve_options* solve,
                            tg_fixed_design_analysis* out, double* von_mises_out,
                            double* stress_out, double* displacement_out) {
  return guarded([&] {
    validate_grid(grid);
    if (!density || !out) raise(TG_EINVAL, "density and out must be non-null");
    validate_strength(strength);
    auto aj = solve_only_job(grid, params, bcs, nbc, loads, nloads, cg_tolerance,
                             cg_max_iterations, solve);
    analyze_on_job(aj.get(), density, grid->tags, *strength, out, von_mises_out, stress_out,
                   displacement_out);
  });
}

int64_t tg_self_weight_loads(const tg_grid* grid, const uint8_t* mask, double density,
                             double gravity, const double direction[3], tg_nodal_load* out,
                             int64_t cap) {
  int64_t count = -1;
  const int rc = guarded([&] {
    validate_grid(grid);
    if (!direction) raise(TG_EINVAL, "self_weight_loads: direction is null");
    if (density < 0.0) raise(TG_EINVAL, "self_weight_loads: density must be >= 0");
    if (gravity < 0.0) raise(TG_EINVAL, "self_weight_loads: gravity must be >= 0");
    const double len = std::sqrt(direction[0] * direction[0] + direction[1] * direction[1] +
                                 direction[2] * direction[2]);
    if (!(len > 1e-12)) raise(TG_EINVAL, "self_weight_loads: direction must have non-zero length");
    const double d[3] = {direction[0] / len, direction[1] / len, direction[2] / len};
    const Grid g = Grid::make(grid->nx, grid->ny, grid->nz, grid->spacing);
    const double h = grid->spacing;
    const double per_node = gravity * density * (h * h * h) / 8.0;
    std::vector<double> nodef(size_t(g.ndof), 0.0);
    for (int k = 0; k < g.nz; ++k)
      for (int j = 0; j < g.ny; ++j)
        for (int i = 0; i < g.nx; ++i) {
          const int64_t e = (int64_t(k) * g.ny + j) * g.nx + i;
          if (grid->tags && grid->tags[e] == 0) continue;
          if (mask && mask[e] == 2) continue;  // FrozenVoid weighs nothing
          for (int a = 0; a < 8; ++a) {
            const int ox = (a ^ (a >> 1)) & 1, oy = (a >> 1) & 1, oz = a >> 2;
            const int64_t n = (int64_t(k + oz) * g.nny + (j + oy)) * g.nnx + (i + ox);
            for (int c = 0; c < 3; ++c) nodef[size_t(3 * n + c)] += per_node * d[c];
          }
        }
    count = 0;
    for (int64_t n = 0; n < g.nnodes; ++n)
      for (int c = 0; c < 3; ++c) {
        const double v = nodef[size_t(3 * n + c)];
        if (v == 0.0) continue;
        if (out && count < cap) out[count] = tg_nodal_load{int32_t(n), c, v};
        ++count;
      }
  }, /*device=*/false);
  return rc == TG_OK ? count : -1;
}

int tg_minimize_plastic(const tg_grid* grid, const tg_simp_params* params,
                        const tg_dirichlet_bc* bcs, int32_t nbc, const tg_nodal_load* loads,
                        int32_t nloads, const tg_simp_options* simp, const uint8_t* mask,
                        const tg_ladder_options* ladder, tg_progress_fn progress,
                        void* progress_ctx, const volatile int32_t* cancel,
                        tg_ladder_rung* rungs_out, tg_ladder_result* result, double* design_out,
                        double* phys_out) {
  tg_ladder_result res{};
  res.recommended = -1;
  const int rc = guarded([&] {
    validate_grid(grid);
    if (!simp || !ladder || !rungs_out) raise(TG_EINVAL, "simp, ladder and rungs_out must be non-null");
    // minimize_plastic.cpp:394-452.
    if (ladder->rungs < 1 || !ladder->volume_fractions)
      raise(TG_EINVAL, "minimize_plastic: volume_fraction_ladder is empty");
    const double* vf = ladder->volume_fractions;
    for (int r = 0; r < ladder->rungs; ++r) {
      if (!std::isfinite(vf[r]) || !(vf[r] > 0.0) || !(vf[r] <= 1.0))
        raise(TG_EINVAL, "minimize_plastic: a ladder volume fraction is not in (0, 1]");
      if (r > 0 && !(vf[r] < vf[r - 1]))
        raise(TG_EINVAL, "minimize_plastic: volume_fraction_ladder is not strictly descending");
    }
    const tg_strength_spec& sp = ladder->strength;
    if (!std::isfinite(sp.margin_stop) || sp.margin_stop < 0.0)
      raise(TG_EINVAL, "minimize_plastic: margin_stop must be finite and >= 0");
    validate_strength(&sp);
    const int64_t nv = int64_t(grid->nx) * grid->ny * grid->nz;
    std::vector<uint8_t> all_active;
    if (!mask) {
      all_active.assign(size_t(nv), uint8_t(0));  // every voxel Active
      mask = all_active.data();
    }
    // The analysis runs on the caller's grid (its tags, FrozenVoid voxels still
    // soft elements), built once for the whole ladder.
    auto aj = solve_only_job(grid, params, bcs, nbc, loads, nloads, simp->cg_tolerance,
                             simp->cg_max_iterations, &simp->solve);
    std::vector<double> seed, design(static_cast<size_t>(nv)), phys(static_cast<size_t>(nv));
    for (int r = 0; r < ladder->rungs; ++r) {
      tg_ladder_rung& rg = rungs_out[r];
      std::memset(&rg, 0, sizeof rg);
      rg.volume_fraction = vf[r];
      tg_simp_options opt = *simp;
      opt.volume_fraction = vf[r];
      opt.initial_design = seed.empty() ? nullptr : seed.data();
      const int src = simp_optimize_impl(grid, params, bcs, nbc, loads, nloads, &opt, mask,
                                         progress, progress_ctx, cancel, nullptr, design.data(),
                                         phys.data(), &rg.optimization);
      if (src != TG_OK) throw Error(src, g_err);
      res.evaluated = r + 1;
      if (rg.optimization.cancelled) {  // the terminal rung, unanalysed
        res.cancelled = 1;
        break;
      }
      if (rg.optimization.infeasible || rg.optimization.non_convergent) continue;
      rg.trajectory_ok = 1;
      if (load_path_host(aj->fp.g, grid->tags, phys.data(), sp.printed_iso)) {
        if (ladder->warm_start_inherit)
          seed = phys;
        else
          seed.clear();
      }
      analyze_on_job(aj.get(), phys.data(), grid->tags, sp, &rg.analysis, nullptr, nullptr);
      if (rg.analysis.non_convergent) continue;
      rg.analysed = 1;
      rg.accepted = rg.analysis.accepted;
      if (rg.accepted) {
        res.recommended = r;
        if (design_out) std::memcpy(design_out, design.data(), design.size() * sizeof(double));
        if (phys_out) std::memcpy(phys_out, phys.data(), phys.size() * sizeof(double));
      } else if (!(rg.analysis.margin_effective >= sp.margin_stop)) {
        res.stopped_on_margin = 1;
        break;
      }
    }
  });
  if (result) *result = res;
  return rc;
}

}  // extern "C"
