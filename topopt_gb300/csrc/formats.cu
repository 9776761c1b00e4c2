// formats.cu -- the on-disk formats the reference's post-processing reads:
// design.bin v1 (core/include/topopt/design_store.hpp:40-90; design_store.cpp),
// fields.bin v1 (core/include/topopt/fields.hpp:33-75; core/src/io/fields.cpp)
// and the iterations.csv row (observability.hpp:72-184; observability.cpp:252-331).
// Host code only.  All integers and floats are little-endian in the files; the
// containers are assembled in memory, written to "<path>.part" and renamed onto
// the path, so a concurrent reader sees a whole container or none.
#include <cinttypes>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "tg_internal.h"

namespace {

// Values are appended in little-endian order whatever the host's order.
struct Bytes {
  std::vector<uint8_t> b;
  void u8(uint8_t v) { b.push_back(v); }
  void zeros(int n) { b.insert(b.end(), size_t(n), uint8_t(0)); }
  void u64(uint64_t v) {
    for (int k = 0; k < 8; ++k) b.push_back(uint8_t(v >> (8 * k)));
  }
  void u32(uint32_t v) {
    for (int k = 0; k < 4; ++k) b.push_back(uint8_t(v >> (8 * k)));
  }
  void i32(int32_t v) { u32(uint32_t(v)); }
  void i64(int64_t v) { u64(uint64_t(v)); }
  void f64(double v) {
    uint64_t u;
    std::memcpy(&u, &v, 8);
    u64(u);
  }
  void f32(float v) {
    uint32_t u;
    std::memcpy(&u, &v, 4);
    u32(u);
  }
};

struct Reader {
  const std::vector<uint8_t>& b;
  size_t at = 0;
  void need(size_t n) const {
    if (at + n > b.size())
      throw tg::Error(TG_EINVAL, "design.bin: truncated container (wanted " + std::to_string(n) +
                                     " more bytes at offset " + std::to_string(at) + " of " +
                                     std::to_string(b.size()) + ")");
  }
  uint64_t u64() {
    need(8);
    uint64_t v = 0;
    for (int k = 0; k < 8; ++k) v |= uint64_t(b[at + size_t(k)]) << (8 * k);
    at += 8;
    return v;
  }
  uint32_t u32() {
    need(4);
    uint32_t v = 0;
    for (int k = 0; k < 4; ++k) v |= uint32_t(b[at + size_t(k)]) << (8 * k);
    at += 4;
    return v;
  }
  uint8_t u8() {
    need(1);
    return b[at++];
  }
  void skip(size_t n) {
    need(n);
    at += n;
  }
  int32_t i32() { return int32_t(u32()); }
  int64_t i64() { return int64_t(u64()); }
  double f64() {
    const uint64_t u = u64();
    double v;
    std::memcpy(&v, &u, 8);
    return v;
  }
};

constexpr uint8_t kDesignVersion = 1;  // design_store.hpp:95
constexpr uint8_t kFieldsVersion = 1;  // fields.hpp:84

uint64_t fnv1a(const double* d, int64_t n) {
  uint64_t h = 1469598103934665603ULL;  // FNV-1a 64 offset basis
  for (int64_t e = 0; e < n; ++e) {
    uint64_t u;
    std::memcpy(&u, &d[e], 8);
    for (int k = 0; k < 8; ++k) {
      h ^= (u >> (8 * k)) & 0xffu;
      h *= 1099511628211ULL;  // FNV-1a 64 prime
    }
  }
  return h;
}

void publish(const std::string& path, const std::vector<uint8_t>& bytes, const char* what) {
  const std::string tmp = path + ".part";
  std::FILE* f = std::fopen(tmp.c_str(), "wb");
  if (!f) throw tg::Error(TG_EINVAL, std::string("cannot open ") + what + " for writing: " + tmp);
  const size_t n = std::fwrite(bytes.data(), 1, bytes.size(), f);
  const bool ok = n == bytes.size() && std::fflush(f) == 0;
  std::fclose(f);
  if (!ok) {
    std::remove(tmp.c_str());
    throw tg::Error(TG_EINVAL, std::string("failed writing ") + what + ": " + tmp);
  }
  if (std::rename(tmp.c_str(), path.c_str()) != 0) {
    std::remove(tmp.c_str());
    throw tg::Error(TG_EINVAL, std::string("failed publishing ") + what + ": " + path);
  }
}

void frame_header(Bytes& w, uint8_t version, const tg_grid_frame& g) {
  w.u8(version);
  w.zeros(3);
  w.i32(g.nx);
  w.i32(g.ny);
  w.i32(g.nz);
  w.f64(g.origin[0]);
  w.f64(g.origin[1]);
  w.f64(g.origin[2]);
  w.f64(g.spacing);
}

template <class F>
int host_call(F&& fn) {
  try {
    fn();
    return TG_OK;
  } catch (const tg::Error& e) {
    tg::set_last_error(e.what());
    return e.code;
  } catch (const std::exception& e) {
    tg::set_last_error(e.what());
    return TG_EINVAL;
  }
}

void check_frame(const tg_grid_frame* f) {
  if (!f || f->nx < 1 || f->ny < 1 || f->nz < 1)
    throw tg::Error(TG_EINVAL, "grid frame must have positive dimensions");
}

}  // namespace

extern "C" {

uint64_t tg_design_fingerprint(const double* density, int64_t count) {
  return density && count > 0 ? fnv1a(density, count) : fnv1a(nullptr, 0);
}

int32_t tg_write_design_file(const char* path, const tg_grid_frame* frame,
                             const tg_design_variant* variants, int32_t count) {
  int32_t written = -1;
  const int rc = host_call([&] {
    check_frame(frame);
    if (!path || count < 0 || (count > 0 && !variants))
      throw tg::Error(TG_EINVAL, "design.bin: path, count and variants are required");
    const int64_t nv = int64_t(frame->nx) * frame->ny * frame->nz;
    // Blocks are the variants that carry a density (design_store.cpp: "every
    // evaluated variant with a field").
    std::vector<const tg_design_variant*> blocks;
    for (int32_t i = 0; i < count; ++i)
      if (variants[i].density) blocks.push_back(&variants[i]);
    Bytes w;
    frame_header(w, kDesignVersion, *frame);
    w.i32(int32_t(blocks.size()));
    w.zeros(4);
    for (const tg_design_variant* v : blocks) {
      w.f64(v->requested_volume_fraction);
      w.f64(v->achieved_volume_fraction);
      w.f64(v->margin_worst_case);
      w.f64(v->margin_effective);
      w.f64(v->max_von_mises);
      w.i32(v->accepted ? 1 : 0);
      w.i32(v->iterations);
      for (int c = 0; c < 3; ++c) w.f64(v->applied_build_dir[c]);
      w.i32(v->build_direction_auto_applied ? 1 : 0);
      w.i32(v->export_baked ? 1 : 0);
      w.u64(fnv1a(v->density, nv));
      w.i64(nv);
      for (int64_t e = 0; e < nv; ++e) w.f64(v->density[e]);
    }
    publish(path, w.b, "design file");
    written = int32_t(blocks.size());
  });
  return rc == TG_OK ? written : -1;
}

int tg_read_design_file(const char* path, tg_grid_frame* frame, int32_t* count,
                        tg_design_variant* variants_out, int32_t cap, double* density_out) {
  return host_call([&] {
    if (!path || !frame || !count) throw tg::Error(TG_EINVAL, "path, frame and count are required");
    std::FILE* f = std::fopen(path, "rb");
    if (!f) throw tg::Error(TG_EINVAL, std::string("cannot open design file: ") + path);
    std::vector<uint8_t> bytes;
    uint8_t buf[1 << 16];
    size_t n;
    while ((n = std::fread(buf, 1, sizeof buf, f)) > 0) bytes.insert(bytes.end(), buf, buf + n);
    std::fclose(f);
    Reader r{bytes};
    const uint8_t version = r.u8();
    if (version != kDesignVersion)
      throw tg::Error(TG_EINVAL, "design.bin: unrecognised version " + std::to_string(int(version)) +
                                     " (this build reads version 1)");
    r.skip(3);
    tg_grid_frame g{};
    g.nx = r.i32();
    g.ny = r.i32();
    g.nz = r.i32();
    for (int c = 0; c < 3; ++c) g.origin[c] = r.f64();
    g.spacing = r.f64();
    const int32_t nblocks = r.i32();
    r.skip(4);
    if (g.nx <= 0 || g.ny <= 0 || g.nz <= 0 || nblocks < 0)
      throw tg::Error(TG_EINVAL, "design.bin: nonsensical header");
    // Every variant stores one density per voxel: a header whose voxel count
    // does not fit in the file is refused before anything is allocated.
    const double nvd = double(g.nx) * double(g.ny) * double(g.nz);
    if (nblocks > 0 && nvd * 8.0 > double(bytes.size()))
      throw tg::Error(TG_EINVAL, "design.bin: truncated container (the header's voxel count " +
                                     std::to_string(nvd) + " exceeds the file)");
    const int64_t nv = nblocks > 0 ? int64_t(nvd) : 0;
    std::vector<double> dens(static_cast<size_t>(nv));
    for (int32_t i = 0; i < nblocks; ++i) {
      tg_design_variant v{};
      v.requested_volume_fraction = r.f64();
      v.achieved_volume_fraction = r.f64();
      v.margin_worst_case = r.f64();
      v.margin_effective = r.f64();
      v.max_von_mises = r.f64();
      v.accepted = r.i32() != 0;
      v.iterations = r.i32();
      for (int c = 0; c < 3; ++c) v.applied_build_dir[c] = r.f64();
      v.build_direction_auto_applied = r.i32() != 0;
      v.export_baked = r.i32() != 0;
      v.fingerprint = r.u64();
      const int64_t cnt = r.i64();
      if (cnt != nv)
        throw tg::Error(TG_EINVAL, "design.bin: variant " + std::to_string(i) + " density count " +
                                       std::to_string(cnt) + " != header voxel count " +
                                       std::to_string(nv));
      for (int64_t e = 0; e < nv; ++e) dens[size_t(e)] = r.f64();
      if (fnv1a(dens.data(), nv) != v.fingerprint)
        throw tg::Error(TG_EINVAL, "design.bin: variant " + std::to_string(i) +
                                       " density does not match its recorded fingerprint");
      if (i < cap && variants_out && density_out) {
        double* dst = density_out + size_t(i) * size_t(nv);
        std::memcpy(dst, dens.data(), size_t(nv) * sizeof(double));
        v.density = dst;
        variants_out[i] = v;
      }
    }
    *frame = g;
    *count = nblocks;
  });
}

int32_t tg_write_fields_file(const char* path, const tg_grid_frame* frame,
                             const tg_fields_variant* variants, int32_t count) {
  int32_t written = -1;
  const int rc = host_call([&] {
    check_frame(frame);
    if (!path || count < 0 || (count > 0 && !variants))
      throw tg::Error(TG_EINVAL, "fields.bin: path, count and variants are required");
    const int64_t nv = int64_t(frame->nx) * frame->ny * frame->nz;
    const int64_t nn = int64_t(frame->nx + 1) * (frame->ny + 1) * (frame->nz + 1);
    Bytes w;
    frame_header(w, kFieldsVersion, *frame);
    const double h = frame->spacing;
    w.f64(h * h * h);  // VoxelGrid::voxel_volume
    w.i32(count);
    w.zeros(4);
    for (int32_t i = 0; i < count; ++i) {
      const tg_fields_variant& v = variants[i];
      if (!v.von_mises || !v.displacement)
        throw tg::Error(TG_EINVAL, "fields.bin: variant " + std::to_string(i) +
                                       " needs its von Mises and displacement fields");
      w.f64(v.requested_volume_fraction);
      w.f64(v.mass_grams);
      w.i32(v.support_volume_voxels);
      w.zeros(4);
      w.i64(nv);
      w.i64(0);  // the stress tensor is absent in v1
      w.i64(3 * nn);
      for (int64_t e = 0; e < nv; ++e) w.f32(static_cast<float>(v.von_mises[e]));
      for (int64_t d = 0; d < 3 * nn; ++d) w.f32(static_cast<float>(v.displacement[d]));
    }
    publish(path, w.b, "fields file");
    written = count;
  });
  return rc == TG_OK ? written : -1;
}

const char* tg_iteration_csv_header(void) {
  return "rung,iter,wall_ms,compliance,achieved_vf,plateau,cg_iters,cg_multigrid,beta,"
         "hier_built,mg_cycles_attempted,infeasible,recycle_dim,active_fraction,"
         "total_ms,tail_prev_ms,filter_ms,project_ms,solve_ms,fea_ms,sens_ms,"
         "update_ms,analysis_ms,observe_ms,residual_ms,"
         "solver_build_ms,mg_build_ms,mg_ms,cg_ms,geneo_setup_ms,geneo_apply_ms,"
         "recycle_ms,"
         "fea_solves,matvecs,geneo_dim,geneo_action,geneo_burn,geneo_threshold,"
         "rss_mb,peak_rss_mb,compressed_mb,available_mb,major_faults,swapins";
}

void tg_iteration_record_from(const tg_simp_iteration* row, int32_t infeasible,
                              tg_iteration_record* out) {
  if (!row || !out) return;
  tg_iteration_record r{};
  r.iteration = row->iteration;
  r.compliance = row->compliance;
  r.volume_fraction = row->volume_fraction;
  r.cg_iterations = row->cg_iterations;
  r.cg_multigrid = row->used_multigrid;
  r.beta = row->beta;
  r.hier_built = row->hier_built;
  r.mg_cycles_attempted = row->mg_cycles_attempted;
  r.infeasible = infeasible;
  // A solve's active fraction is in (0, 1]; a zeroed row carries none (full domain).
  r.active_fraction = row->active_fraction > 0.0 ? row->active_fraction : 1.0;
  r.total_ms = row->t_total_ms;
  r.filter_ms = row->t_filter_ms;
  r.solve_ms = row->t_solve_ms + row->t_sensitivity_ms;
  r.fea_ms = row->t_solve_ms;
  r.sens_ms = row->t_sensitivity_ms;
  r.update_ms = row->t_update_ms;
  r.residual_ms = row->t_total_ms - (row->t_filter_ms + r.solve_ms + row->t_update_ms);
  r.cg_ms = row->t_solve_ms;
  r.fea_solves = 1;
  r.matvecs = row->fine_matvecs + row->fine_matvecs_lowp;
  r.rss_mb = r.peak_rss_mb = r.compressed_mb = r.available_mb = -1.0;
  r.major_faults = r.swapins = -1;
  *out = r;
}

int64_t tg_iteration_csv_row(int64_t rung, const tg_iteration_record* o, int64_t wall_ms,
                             char* buf, int64_t cap) {
  if (!o) return -1;
  char tmp[1024];
  const int n = std::snprintf(
      tmp, sizeof tmp,
      "%" PRId64 ",%d,%lld,%.10g,%.6f,%d,%d,%d,%.6g,%d,%d,%d,%d,%.6f,"
      "%.3f,%.3f,%.3f,%.3f,%.3f,%.3f,%.3f,%.3f,%.3f,%.3f,%.3f,"
      "%.3f,%.3f,%.3f,%.3f,%.3f,%.3f,%.3f,"
      "%lld,%lld,%d,%d,%d,%d,"
      "%.2f,%.2f,%.2f,%.2f,%lld,%lld\n",
      rung, o->iteration, (long long)wall_ms, o->compliance, o->volume_fraction,
      o->plateau ? 1 : 0, o->cg_iterations, o->cg_multigrid ? 1 : 0, o->beta,
      o->hier_built ? 1 : 0, o->mg_cycles_attempted, o->infeasible ? 1 : 0, o->recycle_dim,
      o->active_fraction, o->total_ms, o->tail_prev_ms, o->filter_ms, o->project_ms,
      o->solve_ms, o->fea_ms, o->sens_ms, o->update_ms, o->analysis_ms, o->observe_ms,
      o->residual_ms, o->solver_build_ms, o->mg_build_ms, o->mg_ms, o->cg_ms,
      o->geneo_setup_ms, o->geneo_apply_ms, o->recycle_ms, (long long)o->fea_solves,
      (long long)o->matvecs, o->geneo_dim, o->geneo_action, o->geneo_burn, o->geneo_threshold,
      o->rss_mb, o->peak_rss_mb, o->compressed_mb, o->available_mb, (long long)o->major_faults,
      (long long)o->swapins);
  if (n < 0) return -1;
  if (buf && cap > n) std::memcpy(buf, tmp, size_t(n) + 1);
  return n;
}

}  // extern "C"
