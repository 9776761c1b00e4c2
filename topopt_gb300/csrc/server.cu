// server.cu -- the serving loop: continuous batching of optimisation jobs.
//
// The reference runs one optimisation per driving thread (simp_optimize called
// by minimize_plastic / the app bridge, TopOptBridge.hpp:262-269); this is the
// GB300 form of that caller for many concurrent requests.  Requests are queued
// in arrival order and admitted, head first, when an active slot is free and the
// job's device-memory estimate (tg_job_estimate_bytes) fits in what is left of
// the HBM budget; a request whose estimate exceeds the whole budget is rejected
// at submission.  Each admitted job runs on its own worker thread and its own
// CUDA stream (tg_simp_optimize / tg_simp_optimize_masked: design, displacement
// and multigrid hierarchy resident on the device for all its design
// iterations), so the kernels of the jobs in flight overlap on the GPU.  A job's
// result does not depend on what else is running: every job owns its buffers and
// stream, and every reduction in the library has a fixed order.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "tg_internal.h"

namespace {

double ms_since(const std::chrono::steady_clock::time_point& t0) {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

struct Request {
  int64_t ticket = 0;
  // The problem, copied at submission (the caller's buffers need not outlive it).
  tg_grid grid{};
  std::vector<uint8_t> tags, mask;
  bool has_tags = false, has_mask = false;
  tg_simp_params params{};
  std::vector<tg_dirichlet_bc> bcs;
  std::vector<tg_nodal_load> loads;
  tg_simp_options options{};
  std::vector<tg_projection_stage> stages;  // options.projection, copied
  std::vector<double> seed;                  // options.initial_design, copied
  int64_t estimate = 0;
  std::chrono::steady_clock::time_point t_submit, t_admit, t_done;
  // Outcome.
  bool done = false;
  int status = TG_OK;
  std::string error;
  tg_simp_result result{};
  std::vector<double> design, phys;
};

}  // namespace

struct tg_server {
  tg_server_config cfg{};
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<std::shared_ptr<Request>> pending;
  std::map<int64_t, std::shared_ptr<Request>> tickets;
  std::vector<std::thread> workers;
  int64_t next_ticket = 1;
  int64_t bytes_in_use = 0, peak_bytes = 0;
  int64_t submitted = 0, admitted = 0, completed = 0, rejected = 0;
  int active = 0, peak_active = 0;
  bool stopping = false;
  std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
  double busy_ms = 0.0;  // time with at least one job running
  std::chrono::steady_clock::time_point busy_since;

  void worker() {
    for (;;) {
      std::shared_ptr<Request> r;
      {
        std::unique_lock<std::mutex> lk(mu);
        cv_work.wait(lk, [&] {
          return stopping ||
                 (!pending.empty() && bytes_in_use + pending.front()->estimate <= cfg.hbm_budget_bytes);
        });
        if (stopping) return;
        r = pending.front();
        pending.pop_front();
        bytes_in_use += r->estimate;
        peak_bytes = std::max(peak_bytes, bytes_in_use);
        if (active == 0) busy_since = std::chrono::steady_clock::now();
        ++active;
        peak_active = std::max(peak_active, active);
        ++admitted;
        r->t_admit = std::chrono::steady_clock::now();
      }
      run(*r);
      {
        std::lock_guard<std::mutex> lk(mu);
        bytes_in_use -= r->estimate;
        --active;
        if (active == 0)
          busy_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() -
                                                               busy_since)
                         .count();
        ++completed;
        r->t_done = std::chrono::steady_clock::now();
        r->done = true;
      }
      cv_done.notify_all();
      cv_work.notify_all();  // memory and a slot came free
    }
  }

  void run(Request& r) {
    tg_set_device(cfg.device);
    const int64_t nv = int64_t(r.grid.nx) * r.grid.ny * r.grid.nz;
    r.design.assign(size_t(nv), 0.0);
    r.phys.assign(size_t(nv), 0.0);
    tg_grid g = r.grid;
    g.tags = r.has_tags ? r.tags.data() : nullptr;
    r.options.projection = r.stages.empty() ? nullptr : r.stages.data();
    r.options.initial_design = r.seed.empty() ? nullptr : r.seed.data();
    const int rc =
        r.has_mask
            ? tg_simp_optimize_masked(&g, &r.params, r.bcs.data(), int32_t(r.bcs.size()),
                                      r.loads.data(), int32_t(r.loads.size()), &r.options,
                                      r.mask.data(), nullptr, nullptr, nullptr, nullptr,
                                      r.design.data(), r.phys.data(), &r.result)
            : tg_simp_optimize(&g, &r.params, r.bcs.data(), int32_t(r.bcs.size()),
                               r.loads.data(), int32_t(r.loads.size()), &r.options, nullptr,
                               nullptr, nullptr, nullptr, r.design.data(), r.phys.data(),
                               &r.result);
    r.status = rc;
    if (rc != TG_OK) r.error = tg_last_error();
  }
};

// tg_server_submit after its argument checks: copies the problem and queues it.
static int submit_request(tg_server* s, const tg_grid* grid, const tg_simp_params* params,
                          const tg_dirichlet_bc* bcs, int32_t nbc, const tg_nodal_load* loads,
                          int32_t nloads, const tg_simp_options* options, const uint8_t* mask,
                          int64_t* ticket_out) {
  auto r = std::make_shared<Request>();
  r->grid = *grid;
  const int64_t nv = int64_t(grid->nx) * grid->ny * grid->nz;
  if (grid->tags) {
    r->tags.assign(grid->tags, grid->tags + nv);
    r->has_tags = true;
  }
  if (mask) {
    r->mask.assign(mask, mask + nv);
    r->has_mask = true;
  }
  r->grid.tags = nullptr;
  r->params = *params;
  r->bcs.assign(bcs, bcs + nbc);
  r->loads.assign(loads, loads + nloads);
  r->options = *options;
  if (options->projection && options->projection_stages > 0)
    r->stages.assign(options->projection, options->projection + options->projection_stages);
  r->options.projection = nullptr;
  if (options->initial_design) r->seed.assign(options->initial_design, options->initial_design + nv);
  r->options.initial_design = nullptr;
  r->estimate = tg_job_estimate_bytes(grid, options);
  r->t_submit = std::chrono::steady_clock::now();
  std::lock_guard<std::mutex> lk(s->mu);
  ++s->submitted;
  if (r->estimate <= 0 || r->estimate > s->cfg.hbm_budget_bytes) {
    ++s->rejected;
    tg::set_last_error("tg_server_submit: the job's device-memory estimate exceeds the HBM budget");
    return TG_ENOMEM;
  }
  r->ticket = s->next_ticket++;
  s->tickets[r->ticket] = r;
  s->pending.push_back(r);
  *ticket_out = r->ticket;
  s->cv_work.notify_all();
  return TG_OK;
}

extern "C" {

int tg_server_create(const tg_server_config* cfg, tg_server** out) {
  if (!cfg || !out) {
    tg::set_last_error("tg_server_create: cfg and out must be non-null");
    return TG_EINVAL;
  }
  if (cfg->hbm_budget_bytes <= 0 || cfg->max_active < 1) {
    tg::set_last_error("tg_server_create: hbm_budget_bytes must be > 0 and max_active >= 1");
    return TG_EINVAL;
  }
  std::unique_ptr<tg_server> s;
  try {
    s = std::make_unique<tg_server>();
    s->cfg = *cfg;
    tg_server* sp = s.get();
    for (int i = 0; i < cfg->max_active; ++i) s->workers.emplace_back([sp] { sp->worker(); });
  } catch (const std::exception& e) {
    // The server or a worker thread could not be created: stop and join the
    // workers already running, so that no joinable thread is destroyed.
    if (s) {
      {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stopping = true;
      }
      s->cv_work.notify_all();
      for (std::thread& t : s->workers) t.join();
    }
    tg::set_last_error(std::string("tg_server_create: ") + e.what());
    return TG_ENOMEM;
  }
  *out = s.release();
  return TG_OK;
}

int tg_server_submit(tg_server* s, const tg_grid* grid, const tg_simp_params* params,
                     const tg_dirichlet_bc* bcs, int32_t nbc, const tg_nodal_load* loads,
                     int32_t nloads, const tg_simp_options* options, const uint8_t* mask,
                     int64_t* ticket_out) {
  if (!s || !grid || !params || !options || !ticket_out || nbc < 0 || nloads < 0 ||
      (nbc > 0 && !bcs) || (nloads > 0 && !loads) || grid->nx < 1 || grid->ny < 1 ||
      grid->nz < 1) {
    tg::set_last_error("tg_server_submit: invalid arguments");
    return TG_EINVAL;
  }
  try {
    return submit_request(s, grid, params, bcs, nbc, loads, nloads, options, mask, ticket_out);
  } catch (const std::exception& e) {  // the copies of the problem could not be made
    tg::set_last_error(std::string("tg_server_submit: ") + e.what());
    return TG_ENOMEM;
  }
}

int tg_server_wait(tg_server* s, int64_t ticket, tg_server_result* out, double* design_out,
                   double* phys_out) {
  if (!s) {
    tg::set_last_error("tg_server_wait: server is null");
    return TG_EINVAL;
  }
  std::shared_ptr<Request> r;
  {
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->tickets.find(ticket);
    if (it == s->tickets.end()) {
      tg::set_last_error("tg_server_wait: unknown ticket");
      return TG_EINVAL;
    }
    r = it->second;
    s->cv_done.wait(lk, [&] { return r->done; });
    s->tickets.erase(ticket);  // by key: another waiter on the same ticket may have erased it
  }
  if (out) {
    std::memset(out, 0, sizeof *out);
    out->ticket = r->ticket;
    out->status = r->status;
    out->result = r->result;
    out->estimate_bytes = r->estimate;
    out->t_queue_ms =
        std::chrono::duration<double, std::milli>(r->t_admit - r->t_submit).count();
    out->t_run_ms = std::chrono::duration<double, std::milli>(r->t_done - r->t_admit).count();
    out->t_latency_ms =
        std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count();
  }
  if (design_out) std::memcpy(design_out, r->design.data(), r->design.size() * sizeof(double));
  if (phys_out) std::memcpy(phys_out, r->phys.data(), r->phys.size() * sizeof(double));
  if (r->status != TG_OK) tg::set_last_error(r->error);
  return r->status;
}

int tg_server_stats(tg_server* s, tg_server_counters* out) {
  if (!s || !out) {
    tg::set_last_error("tg_server_stats: null argument");
    return TG_EINVAL;
  }
  std::lock_guard<std::mutex> lk(s->mu);
  std::memset(out, 0, sizeof *out);
  out->submitted = s->submitted;
  out->admitted = s->admitted;
  out->completed = s->completed;
  out->rejected = s->rejected;
  out->queued = int64_t(s->pending.size());
  out->active = s->active;
  out->peak_active = s->peak_active;
  out->bytes_in_use = s->bytes_in_use;
  out->peak_bytes = s->peak_bytes;
  out->uptime_ms = ms_since(s->t0);
  double busy = s->busy_ms;
  if (s->active > 0)
    busy += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() -
                                                      s->busy_since)
                .count();
  out->busy_ms = busy;
  return TG_OK;
}

void tg_server_destroy(tg_server* s) {
  if (!s) return;
  {
    std::unique_lock<std::mutex> lk(s->mu);
    // Queued jobs are dropped (their waiters see TG_EINVAL); admitted ones finish.
    for (auto& r : s->pending) {
      r->status = TG_EINVAL;
      r->error = "tg_server_destroy: the server stopped before the job was admitted";
      r->t_admit = r->t_done = std::chrono::steady_clock::now();
      r->done = true;
    }
    s->pending.clear();
    s->cv_done.notify_all();
    s->cv_done.wait(lk, [&] { return s->active == 0; });
    s->stopping = true;
  }
  s->cv_work.notify_all();
  for (std::thread& t : s->workers) t.join();
  delete s;
}

}  // extern "C"
