// tune.cu -- per-grid schedule table of the FP32 fine operator.
//
// No reference counterpart: the reference's operator has one schedule (colour
// sweeps on a thread pool).  Here the column-blocked FP32 kernel has several
// tile shapes and z-chunk lengths; which one is fastest depends on how the grid
// divides into tiles.  The table maps grid dimensions to the schedule in use.
#include <cuda_runtime.h>

#include <atomic>
#include <map>
#include <mutex>
#include <tuple>

#include "tg_internal.h"

namespace tg {
namespace {

std::mutex g_sched_mu;
std::map<std::tuple<int, int, int>, FineSchedule> g_sched;
bool g_have_override = false;
FineSchedule g_override;

}  // namespace

FineSchedule fine_schedule_for(const Grid& g) {
  std::lock_guard<std::mutex> lk(g_sched_mu);
  if (g_have_override) return g_override;
  auto it = g_sched.find(std::make_tuple(g.nx, g.ny, g.nz));
  if (it != g_sched.end()) return it->second;
  return default_fine_schedule(g);
}

void set_fine_schedule_override(const FineSchedule* s) {
  std::lock_guard<std::mutex> lk(g_sched_mu);
  g_have_override = s != nullptr;
  if (s) g_override = *s;
}

void set_fine_schedule(const Grid& g, const FineSchedule& s) {
  std::lock_guard<std::mutex> lk(g_sched_mu);
  g_sched[std::make_tuple(g.nx, g.ny, g.nz)] = s;
}

namespace {
std::atomic<bool> g_level1_tc{true};
}
bool level1_tc_enabled() { return g_level1_tc.load(); }
void set_level1_tc(bool on) { g_level1_tc.store(on); }

}  // namespace tg
