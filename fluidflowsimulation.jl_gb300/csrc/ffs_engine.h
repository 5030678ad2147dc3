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

class EngineBase {
 public:
  virtual ~EngineBase() {}
  virtual int create(const ffs_params& p, std::string& err) = 0;
  virtual int set_fields(const double* u1, const double* u2, const double* u3, const double* rho, int layout,
                         std::string& err) = 0;
  virtual int initialize(std::string& err) = 0;
  virtual int step(int64_t n, std::string& err) = 0;
  virtual int get_fields(double* u1, double* u2, double* u3, double* rho, int layout, std::string& err) = 0;
  virtual int get_spectral(int comp, double* out, std::string& err) = 0;
  virtual int set_spectral(int comp, const double* in, std::string& err) = 0;
  virtual int time_steps(int64_t n, double* ms, std::string& err) = 0;
  virtual int profile(int64_t n, std::vector<KernelTiming>& out, std::string& err) = 0;
  virtual int launches_per_step() const = 0;
  virtual int64_t device_bytes() const = 0;
  virtual void* stream() const = 0;
  // host-side views
  std::string header;
  int ncols_stats = 0, ncols_rec = 0;
  int lenH = 0, lenV = 0;
  std::vector<double> rec_host;    // drained stats records
  std::vector<double> spec_host;   // drained spectrum records (iteration + 4 spectra)
  int64_t iteration = 0;
  double time = 0.0, dt = 0.0;
  bool initialized = false;
};

EngineBase* make_engine_f32();
EngineBase* make_engine_f64();

}  // namespace ffsgpu
