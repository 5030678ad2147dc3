// C ABI of libffs (declared in include/ffs.h). No C++ exception crosses this file.
#include <string.h>

#include <memory>
#include <string>

#include "ffs_engine.h"

struct ffs_handle {
  ffs_params p;
  std::unique_ptr<ffsgpu::EngineBase> eng;
  std::string err;
};

namespace {
thread_local std::string g_create_err;
}  // namespace

namespace ffsgpu {
// message for ffs_last_error(NULL) from entry points that have no handle
void set_global_error(const std::string& msg) { g_create_err = msg; }
}  // namespace ffsgpu

namespace {

template <typename F> int guarded(ffs_handle* h, F&& f) {
  if (!h) return FFS_EINVAL;
  try {
    return f();
  } catch (const std::exception& e) {
    h->err = std::string("internal error: ") + e.what();
    return FFS_EINVAL;
  } catch (...) {
    h->err = "internal error";
    return FFS_EINVAL;
  }
}
}  // namespace

extern "C" {

int ffs_params_default(ffs_params* p) {
  if (!p) return FFS_EINVAL;
  memset(p, 0, sizeof(*p));
  p->nx = p->ny = p->nz = 32;
  p->lx = p->ly = p->lz = 1.0;
  p->nu = 0.0;
  p->cutoff = 2.0 / 3.0;                 // Globals.jl:132
  p->integrator = FFS_ETD3;              // simulationtypes.jl:308
  p->variable_dt = 1;                    // simulationtypes.jl:309
  p->cfl = 0.18;                         // simulationtypes.jl:310
  p->dt = 0.0;                           // simulationtypes.jl:311
  p->hv_m = 2;                           // simulationtypes.jl:300
  p->smag_c = 0.17;                      // les_types.jl:365
  p->filter_width = 0.0;                 // les_types.jl:366 default
  p->density_pr = 1.0;
  p->gravity_dir = 2;                    // density_stratification_types.jl:153
  p->forcing_power = 0.1;
  p->forcing_kf = 2.5;
  p->precision = FFS_FP64;
  p->dt_stat = 1;
  p->dt_spec = 1;
  p->write_time = 1 << 30;
  p->reference_cfl_slot = 1;
  p->stats_capacity = 256;
  p->spec_capacity = 16;
  p->kernel_variant = 0;
  p->autotune = 0;
  return FFS_OK;
}

int ffs_create(const ffs_params* p, ffs_handle** out) {
  if (!p || !out) return FFS_EINVAL;
  *out = nullptr;
  ffs_handle* h = nullptr;
  try {
    h = new ffs_handle();
    h->p = *p;
    if (p->precision == FFS_FP32) h->eng.reset(ffsgpu::make_engine_f32());
    else if (p->precision == FFS_FP64) h->eng.reset(ffsgpu::make_engine_f64());
    else { g_create_err = "precision must be FFS_FP64 or FFS_FP32"; delete h; return FFS_EINVAL; }
    int rc = h->eng->create(*p, h->err);
    if (rc) { g_create_err = h->err; delete h; return rc; }
  } catch (...) {
    g_create_err = "allocation failure in ffs_create";
    delete h;
    return FFS_ENOMEM;
  }
  *out = h;
  return FFS_OK;
}

int ffs_set_fields(ffs_handle* h, const double* u1, const double* u2, const double* u3, const double* rho,
                   int32_t layout) {
  return guarded(h, [&] { return h->eng->set_fields(u1, u2, u3, rho, layout, h->err); });
}

int ffs_initialize(ffs_handle* h) {
  return guarded(h, [&] { return h->eng->initialize(h->err); });
}

int ffs_step(ffs_handle* h, int64_t nsteps) {
  return guarded(h, [&] { return h->eng->step(nsteps, h->err); });
}

int ffs_forcing_shells(const ffs_handle* h) { return h ? h->eng->forcing_shells() : FFS_EINVAL; }

int ffs_forcing_array(ffs_handle* h, int32_t which, double* v, int32_t n, int32_t set) {
  return guarded(h, [&] { return h->eng->forcing_array(which, v, n, set, h->err); });
}

int ffs_finalize(ffs_handle* h) {
  return guarded(h, [&] { return h->eng->finish(h->err); });
}

int ffs_capture_output(ffs_handle* h, int32_t on) {
  return guarded(h, [&] { return h->eng->capture_output(on, h->err); });
}

int ffs_output_field(ffs_handle* h, int32_t field, double* out, int64_t* iteration) {
  if (!out) return FFS_EINVAL;
  return guarded(h, [&] { return h->eng->output_field(field, out, iteration, h->err); });
}

int ffs_get_fields(ffs_handle* h, double* u1, double* u2, double* u3, double* rho, int32_t layout) {
  return guarded(h, [&] { return h->eng->get_fields(u1, u2, u3, rho, layout, h->err); });
}

int ffs_get_spectral(ffs_handle* h, int32_t comp, double* out) {
  if (!out) return FFS_EINVAL;
  return guarded(h, [&] { return h->eng->get_spectral(comp, out, h->err); });
}

int ffs_set_spectral(ffs_handle* h, int32_t comp, const double* in) {
  if (!in) return FFS_EINVAL;
  return guarded(h, [&] { return h->eng->set_spectral(comp, in, h->err); });
}

int ffs_stats_header(const ffs_handle* h, char* buf, int64_t len) {
  if (!h || !buf || len <= 0) return FFS_EINVAL;
  const std::string& s = h->eng->header;
  if ((int64_t)s.size() + 1 > len) return FFS_EINVAL;
  memcpy(buf, s.c_str(), s.size() + 1);
  return FFS_OK;
}

int32_t ffs_stats_ncols(const ffs_handle* h) { return h ? h->eng->ncols_stats : FFS_EINVAL; }
int32_t ffs_record_ncols(const ffs_handle* h) { return h ? h->eng->ncols_rec : FFS_EINVAL; }

int64_t ffs_stats_records(ffs_handle* h, double* out, int64_t max_rows) {
  if (!h) return FFS_EINVAL;
  auto& v = h->eng->rec_host;
  const int64_t nc = h->eng->ncols_rec;
  const int64_t have = (int64_t)v.size() / nc;
  if (!out) return have;
  const int64_t n = max_rows < have ? max_rows : have;
  memcpy(out, v.data(), sizeof(double) * n * nc);
  v.erase(v.begin(), v.begin() + n * nc);
  return n;
}

int ffs_stats(ffs_handle* h, double* row, int32_t ncols) {
  if (!h || !row) return FFS_EINVAL;
  const auto& r = h->eng->last_rec;
  if (r.empty()) {
    h->err = "no stats record yet (stats are taken at iterations that are multiples of dtStat)";
    return FFS_ESTATE;
  }
  if (ncols < h->eng->ncols_stats) {
    h->err = "row buffer shorter than the Stats.txt columns";
    return FFS_EINVAL;
  }
  memcpy(row, r.data(), sizeof(double) * h->eng->ncols_stats);
  return FFS_OK;
}

int ffs_spectrum(ffs_handle* h, double* specH, double* specV, int64_t lenH, int64_t lenV) {
  if (!h || !specH || !specV) return FFS_EINVAL;
  if (lenH != h->eng->lenH || lenV != h->eng->lenV) {
    h->err = "spectrum lengths differ from ffs_spectrum_lengths";
    return FFS_EINVAL;
  }
  return guarded(h, [&] { return h->eng->spectrum_u(specH, specV, h->err); });
}

int ffs_spectrum_lengths(const ffs_handle* h, int32_t* lenH, int32_t* lenV) {
  if (!h || !lenH || !lenV) return FFS_EINVAL;
  *lenH = h->eng->lenH;
  *lenV = h->eng->lenV;
  return FFS_OK;
}

int ffs_spectrum_fields(const ffs_handle* h, char* buf, int64_t len) {
  if (!h || !buf || len <= 0) return FFS_EINVAL;
  const std::string& s = h->eng->spec_names;
  if ((int64_t)s.size() + 1 > len) return FFS_EINVAL;
  memcpy(buf, s.c_str(), s.size() + 1);
  return h->eng->nspecf;
}

int64_t ffs_spectrum_records(ffs_handle* h, double* out, int64_t max_rows) {
  if (!h) return FFS_EINVAL;
  auto& v = h->eng->spec_host;
  const int64_t rl = 1 + (int64_t)h->eng->nspecf * ((int64_t)h->eng->lenH + (int64_t)h->eng->lenV);
  const int64_t have = (int64_t)v.size() / rl;
  if (!out) return have;
  const int64_t n = max_rows < have ? max_rows : have;
  memcpy(out, v.data(), sizeof(double) * n * rl);
  v.erase(v.begin(), v.begin() + n * rl);
  return n;
}

int64_t ffs_iteration(const ffs_handle* h) { return h ? h->eng->iteration : 0; }
double ffs_time(const ffs_handle* h) { return h ? h->eng->time : 0.0; }
double ffs_dt(const ffs_handle* h) { return h ? h->eng->dt : 0.0; }

int ffs_time_steps(ffs_handle* h, int64_t nsteps, double* ms) {
  if (!ms) return FFS_EINVAL;
  return guarded(h, [&] { return h->eng->time_steps(nsteps, ms, h->err); });
}

int ffs_profile_kernels(ffs_handle* h, int64_t nsteps, char* names, int64_t names_len, double* ms, int32_t max_k,
                        int32_t* nk) {
  if (!names || !ms || !nk) return FFS_EINVAL;
  return guarded(h, [&] {
    std::vector<ffsgpu::KernelTiming> t;
    int rc = h->eng->profile(nsteps, t, h->err);
    if (rc) return rc;
    std::string joined;
    int k = 0;
    for (auto& e : t) {
      if (k >= max_k) break;
      if (k) joined += ",";
      joined += e.name;
      ms[k++] = e.ms;
    }
    if ((int64_t)joined.size() + 1 > names_len) { h->err = "names buffer too small"; return FFS_EINVAL; }
    memcpy(names, joined.c_str(), joined.size() + 1);
    *nk = k;
    return FFS_OK;
  });
}

int32_t ffs_launches_per_step(const ffs_handle* h) { return h ? h->eng->launches_per_step() : 0; }
int64_t ffs_device_bytes(const ffs_handle* h) { return h ? h->eng->device_bytes() : 0; }

int ffs_tuning_report(const ffs_handle* h, char* buf, int64_t len) {
  if (!h || !buf || len <= 0) return FFS_EINVAL;
  const std::string s = h->eng->tuning();
  if ((int64_t)s.size() + 1 > len) return FFS_EINVAL;
  memcpy(buf, s.c_str(), s.size() + 1);
  return FFS_OK;
}
void* ffs_stream(const ffs_handle* h) { return h ? h->eng->stream() : nullptr; }

const char* ffs_last_error(const ffs_handle* h) {
  if (!h) return g_create_err.c_str();
  return h->err.c_str();
}

void ffs_destroy(ffs_handle* h) { delete h; }

}  // extern "C"
