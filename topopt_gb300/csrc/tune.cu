// tune.cu -- per-grid schedule table of the FP32 fine operator.
//
// No reference counterpart: the reference's operator has one schedule (colour
// sweeps on a thread pool).  Here the column-blocked FP32 kernel has several
// tile shapes and z-chunk lengths; which one is fastest depends on how the grid
// divides into tiles.  The table maps grid dimensions to the schedule in use.
#include <cuda_runtime.h>

#include <atomic>
#include <algorithm>
#include <map>
#include <vector>
#include <mutex>
#include <tuple>

#include "tg_internal.h"

namespace tg {
namespace {

std::mutex g_sched_mu;
// (nx, ny, nz, mode): the apply, residual and smoothing modes read different
// vectors and are tuned separately.
std::map<std::tuple<int, int, int, int>, FineSchedule> g_sched;
// One measured sweep at a time.  A grid's entries are published together once
// its sweep ends and are never replaced by a later sweep, so concurrent jobs of
// the same grid (which wait here while it is measured) all run one schedule.
std::mutex g_tune_mu;

struct EventPair {
  cudaEvent_t a = nullptr, b = nullptr;
  EventPair() {
    TG_CUDA(cudaEventCreate(&a));
    TG_CUDA(cudaEventCreate(&b));
  }
  ~EventPair() {
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
  }
};
bool g_have_override = false;
FineSchedule g_override;

}  // namespace

FineSchedule fine_schedule_for(const Grid& g, int mode) {
  std::lock_guard<std::mutex> lk(g_sched_mu);
  if (g_have_override) return g_override;
  auto it = g_sched.find(std::make_tuple(g.nx, g.ny, g.nz, mode));
  if (it != g_sched.end()) return it->second;
  return default_fine_schedule(g);
}

void set_fine_schedule_override(const FineSchedule* s) {
  std::lock_guard<std::mutex> lk(g_sched_mu);
  g_have_override = s != nullptr;
  if (s) g_override = *s;
}

bool fine_schedule_known(const Grid& g) {
  std::lock_guard<std::mutex> lk(g_sched_mu);
  return g_have_override || g_sched.count(std::make_tuple(g.nx, g.ny, g.nz, int(kApply))) != 0;
}

// The measured sweep: every column tile shape with z-chunks of about 8 .. 33
// element layers, and the pencil kernel, each launched once untimed and then
// timed over `reps` back-to-back launches, for each of the three modes as the
// mixed solve runs them: the apply with the kept mask and the p.Ap partials,
// the residual, and the smoothing sweep with its b.y partials (b, invdiag:
// any finite vectors).  The fastest per mode goes into the table for g's
// dimensions, unless another sweep of the same grid published first.  Results
// of every candidate agree to FP32 rounding, so the choice changes timing only.
// Returns the apply's schedule in the table.
FineSchedule autotune_fine_schedule(const Grid& g, const ModalConsts& mc, const float* ef,
                                    const uint8_t* kept, const uint8_t* kn, const float* x,
                                    float* y, double* part, cudaStream_t s, const float* b,
                                    const float* invdiag, int reps) {
  std::lock_guard<std::mutex> tune_lock(g_tune_mu);
  if (fine_schedule_known(g)) return fine_schedule_for(g, kApply);
  std::vector<FineSchedule> cands;
  FineSchedule pencil;
  pencil.kind = FineSchedule::kPencil;
  cands.push_back(pencil);
  std::vector<int> kzs;
  for (int target : {8, 11, 13, 16, 22, 26, 33}) {
    const int chunks = std::max(1, (g.nnz + target - 1) / target);
    const int kz = std::max(8, (g.nnz + chunks - 1) / chunks);
    if (std::find(kzs.begin(), kzs.end(), kz) == kzs.end()) kzs.push_back(kz);
  }
  for (int sh = 0; sh < fine_schedule_shapes(); ++sh)
    for (int kz : kzs) {
      FineSchedule c;
      c.kind = FineSchedule::kColumn;
      c.shape = sh;
      c.kz = kz;
      cands.push_back(c);
    }
  EventPair ev;
  const cudaEvent_t ea = ev.a, eb = ev.b;
  std::vector<std::pair<int, FineSchedule>> chosen;
  for (int mode : {int(kApply), int(kResidual), int(kSmooth)}) {
    if (mode != kApply && (b == nullptr || invdiag == nullptr)) continue;
    const float* bb = mode == kApply ? nullptr : b;
    const float* dd = mode == kSmooth ? invdiag : nullptr;
    double* pp = mode == kResidual ? nullptr : part;
    FineSchedule best = default_fine_schedule(g);
    float best_ms = 1e30f;
    for (const FineSchedule& c : cands) {
      launch_fine_op_sched(c, mode, g, mc, ef, kept, x, bb, dd, 0.6f, y, pp, nullptr, s, kn);
      TG_CUDA(cudaEventRecord(ea, s));
      for (int r = 0; r < reps; ++r)
        launch_fine_op_sched(c, mode, g, mc, ef, kept, x, bb, dd, 0.6f, y, pp, nullptr, s, kn);
      TG_CUDA(cudaEventRecord(eb, s));
      TG_CUDA(cudaEventSynchronize(eb));
      float ms = 0.0f;
      TG_CUDA(cudaEventElapsedTime(&ms, ea, eb));
      if (ms < best_ms) {
        best_ms = ms;
        best = c;
      }
    }
    chosen.emplace_back(mode, best);
  }
  {
    std::lock_guard<std::mutex> lk(g_sched_mu);
    for (const auto& [mode, sch] : chosen)
      g_sched.emplace(std::make_tuple(g.nx, g.ny, g.nz, mode), sch);
  }
  return fine_schedule_for(g, kApply);
}

namespace {
std::atomic<bool> g_level1_tc{true};
}
bool level1_tc_enabled() { return g_level1_tc.load(); }
void set_level1_tc(bool on) { g_level1_tc.store(on); }
namespace {
std::atomic<bool> g_level1_galerkin_fast{true};
}
bool level1_galerkin_fast_enabled() { return g_level1_galerkin_fast.load(); }
void set_level1_galerkin_fast(bool on) { g_level1_galerkin_fast.store(on); }
// Off by default: on the 256x128x128 cantilever the cluster launch took 155 us
// per V-cycle for levels 4..6 against 139 us as separate launches (a fused phase
// costs ~9 us: one cluster of 16 SMs, L2 round trips on every phase).
namespace {
std::atomic<bool> g_coarse_fused{false};
}
bool coarse_fused_enabled() { return g_coarse_fused.load(); }
void set_coarse_fused(bool on) { g_coarse_fused.store(on); }

}  // namespace tg
