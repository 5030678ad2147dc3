// Precision-independent interface between the C ABI and the templated engine.
#pragma once
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/ffs.h"

namespace ffsgpu {

struct KernelTiming {
  std::string name;
  double ms;
};

// Work of one simulation in a batched step (see ffs_batch.cuh), filled by batch_export.
struct BatchGeom {
  int nx, ny, nz;
  int nin, nout;          // fields of the inverse / forward passes
  int kx_tiles;           // KXP / TX of the y and z passes
  int nyr;                // retained ky count
  int yz_groups;          // ny * nz / lyz (x pass CTAs)
  int fwd_z_tiles;        // KXP / txz
  int les, density, etd;
  int table_blocks;       // ETD table CTAs (0: AB3)
  int nparts, upd_blocks; // stats and update CTAs
  int txy, txz, lyz;
  int xfused;             // n of the engine's register-fused x pass (0: none)
  int kxp;                // padded kx row length (tiles of a size class: kxp / tile)
};

class EngineBase {
 public:
  virtual ~EngineBase() {}
  virtual int create(const ffs_params& p, std::string& err) = 0;
  virtual int set_fields(const double* u1, const double* u2, const double* u3, const double* rho, int layout,
                         std::string& err) = 0;
  virtual int initialize(std::string& err) = 0;
  virtual int step(int64_t n, std::string& err) = 0;
  // run_simulation's tail: rhs, forcing and a stats record at the current iteration
  virtual int finish(std::string& err) = 0;
  // kz = 0 plane forcing state per 2D shell (0: R, 1: Em, 2: avgK)
  virtual int forcing_shells() const = 0;
  virtual int forcing_array(int which, double* v, int n, int set, std::string& err) = 0;
  virtual int get_fields(double* u1, double* u2, double* u3, double* rho, int layout, std::string& err) = 0;
  virtual int get_spectral(int comp, double* out, std::string& err) = 0;
  // u spectrum of the current state: H (lenH) horizontal bins, V (lenV) vertical bins
  virtual int spectrum_u(double* H, double* V, std::string& err) = 0;
  virtual int set_spectral(int comp, const double* in, std::string& err) = 0;
  virtual int time_steps(int64_t n, double* ms, std::string& err) = 0;
  virtual int profile(int64_t n, std::vector<KernelTiming>& out, std::string& err) = 0;
  virtual int launches_per_step() const = 0;
  virtual int64_t device_bytes() const = 0;
  virtual void* stream() const = 0;
  // batched stepping: the simulation's parameter block (a BatchInst<T>) and its geometry
  virtual int batch_export(void* bi, size_t bi_size, BatchGeom* g, std::string& err) const = 0;
  // the simulation's own stream waits for an event of another stream
  virtual int stream_wait(void* event, std::string& err) = 0;
  // reuse the buffers for new physics parameters on the same grid and model
  virtual int repurpose(const ffs_params& p, std::string& err) = 0;
  // state after batched steps advanced the simulation outside step()
  virtual int sync_host_state(int64_t it_first, int64_t it_last, std::string& err) = 0;
  // launch shapes picked by the autotuner, with the timings of the candidates
  virtual std::string tuning() const = 0;
  // output capture: the LES fields writeoutput writes at output steps and at the tail
  virtual int capture_output(int on, std::string& err) = 0;
  virtual int output_field(int field, double* out, int64_t* iteration, std::string& err) = 0;
  // host-side views
  std::string header;
  int ncols_stats = 0, ncols_rec = 0;
  int lenH = 0, lenV = 0;
  int nspecf = 4;                  // spectrum fields per record
  std::string spec_names;          // their names, comma-separated
  std::vector<double> rec_host;    // drained stats records
  std::vector<double> last_rec;    // the most recent stats record (kept when rec_host is read)
  std::vector<double> spec_host;   // drained spectrum records (iteration + 4 spectra)
  int64_t iteration = 0;
  double time = 0.0, dt = 0.0;
  bool initialized = false;
};

EngineBase* make_engine_f32();
EngineBase* make_engine_f64();
// device bytes an FP32 engine allocates for these parameters (before creating it)
int64_t estimate_bytes_f32(const ffs_params& p);

}  // namespace ffsgpu
