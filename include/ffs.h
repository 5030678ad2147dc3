/*
 * ffs.h — C ABI of the GB300 pseudo-spectral solver-step engine (libffs.so).
 *
 * The engine replaces the body of FluidFlowSimulation.jl's time loop: the reference's
 * `initialize!(s)` (src/FluidFlowSimulation.jl:67-91) and `advance_in_time!(s)`
 * (src/models.jl:3-17) with everything they call. The reference has no FFI of its own
 * (it extends through Julia multiple dispatch on the Simulation type parameters,
 * src/simulationtypes.jl:45-100); these entry points are what a `ccall` shim mirroring
 * `run_simulation()` (src/FluidFlowSimulation.jl:23-65) binds.
 *
 * Conventions: plain C types only; every function returns 0 on success or a negative
 * FFS_E* code, with a message in ffs_last_error(). No exceptions or aborts cross the
 * ABI. A handle is used by one host thread at a time; handles are independent and
 * each owns a CUDA stream and all of its device memory. The library keeps no pointer
 * to caller memory after a call returns.
 *
 * Field layout (same as the reference's PaddedArray, src/output.jl:6-8): Float64,
 * x fastest, either unpadded nx*ny*nz (layout 0) or padded 2*(nx/2+1)*ny*nz (layout 1).
 */
#ifndef FFS_H
#define FFS_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FFS_OK 0
#define FFS_EINVAL (-1)
#define FFS_ENOMEM (-2)
#define FFS_ECUDA (-3)
#define FFS_ENAN (-4)
#define FFS_ETIMEDOUT (-5)
#define FFS_EUNSUPPORTED (-6)
#define FFS_ESTATE (-7)
#define FFS_ECANCELED (-8)

#define FFS_ETD3 0 /* ETD3rdO (src/time_step_functions/ETD.jl) */
#define FFS_AB3 1  /* Adams_Bashforth3rdO (src/time_step_functions/Adams_Bashforth.jl) */
#define FFS_EULER 2 /* Euller (src/time_step_functions/Euller.jl): u += dt rhs, explicit viscosity */

#define FFS_FP64 0
#define FFS_FP32 1

typedef struct ffs_handle ffs_handle;

/* Mirrors the in-scope keys of the `global` file read by parameters()
 * (src/simulationtypes.jl:242-365, src/Globals.jl:106-183). */
typedef struct ffs_params {
  int32_t nx, ny, nz;          /* nx ny nz */
  double lx, ly, lz;           /* xDomainSize.. in units of 2 pi: k = i / L */
  double nu;                   /* kinematicViscosity */
  double cutoff;               /* cutoff (dealias ratio), default 2/3 */
  int32_t integrator;          /* velocityTimeStep: FFS_ETD3 | FFS_AB3 | FFS_EULER */
  int32_t variable_dt;         /* variableTimestepFlag (default 1) */
  double cfl;                  /* cfl, default 0.18 */
  double dt;                   /* dt (fixed dt, or the initial value) */
  int32_t hyperviscosity;      /* hyperViscosity present */
  double hv_nu;                /* hyperViscosityCoefficient */
  int32_t hv_m;                /* hyperViscosityM, default 2 */
  int32_t les;                 /* lesModel Smagorinsky */
  double smag_c;               /* smagorinskyConstant, default 0.17 */
  double filter_width;         /* filterWidth (<= 0: reference default (lx 2pi/nx)/cutoff) */
  int32_t density;             /* densityStratification */
  double density_pr;           /* Pr */
  double density_gradient;     /* densityGradient */
  double gravity;              /* zAcceleration / referenceDensity */
  int32_t gravity_dir;         /* gravityDirection: 0 x, 1 y, 2 z */
  int32_t forcing;             /* forcing isotropicBand (no reference counterpart) */
  double forcing_power;        /* forcingPower (epsilon) */
  double forcing_kf;           /* forcingKf */
  int32_t precision;           /* FFS_FP64 | FFS_FP32 */
  int32_t dt_stat;             /* dtStat */
  int32_t dt_spec;             /* dtSpec */
  int32_t write_time;          /* writeTime */
  int64_t start;               /* start */
  double start_time;           /* startTime */
  int32_t device;              /* CUDA device ordinal */
  int32_t reference_cfl_slot;  /* 1: CFL uses the reference's reused reduction slot */
  int32_t stats_capacity;      /* stats records kept on the device between reads */
  int32_t spec_capacity;       /* spectrum records kept on the device between reads */
  int32_t kernel_variant;      /* 0: specialised FP32 kernels where available (register-fused x pass,
                                  compile-time FFT lengths); 1: runtime-plan kernels only;
                                  2: as 0 with every compile-time y/z pass on line pairs (packed FP32);
                                  3: as 0 with every compile-time y/z pass one line per thread;
                                  4: as 3 with TX/2 kx lines a CTA in the y/z passes (compile-time
                                  plans at 512 and 1024) */
  int32_t autotune;            /* 1: time the candidate launch shapes at create, keep the fastest */
  int32_t les_model;           /* with les != 0, the eddy-viscosity model of lesModel (les_types.jl:360-395):
                                  FFS_LES_SMAGORINSKY, FFS_LES_VREMAN, FFS_LES_PRODUCTION, FFS_LES_SILVIS,
                                  FFS_LES_STABLE_NL, FFS_LES_DYNAMIC, FFS_LES_PIOMELLI; smag_c holds the
                                  constant of the pointwise models */
  double les_cp;               /* silvisPConstant (Silvis model) */
  double sandp_cb;             /* lesModel SandP: pConstant of the P tensor term (0: none) */
  int32_t passive_scalar;      /* passiveScalar (simulationtypes.jl:198-213, :320-352): a scalar phi
                                  transported like the density, without buoyancy; the fourth
                                  field of ffs_set_fields / ffs_get_fields (scalar.N files) */
  double scalar_pr;            /* scalarPr: diffusivity nu / scalarPr */
  double scalar_gradient;      /* scalarGradient: mean gradient d phi / d(direction) */
  int32_t scalar_dir;          /* scalarDirection: 0 x, 1 y, 2 z */
  int32_t plane_forcing;       /* the reference's kz = 0 plane forcing (forcing_types.jl:335-450):
                                  FFS_PF_RF (rfForcing), FFS_PF_CRF (cRfForcing), FFS_PF_QF (QfForcing),
                                  FFS_PF_NRF (nRfForcing), FFS_PF_CNRF (cNRfForcing), FFS_PF_A (aForcing) */
  double pf_tf;                /* TF */
  double pf_alpha;             /* alphac */
  double pf_kf;                /* kf */
  int32_t pf_zf_tanh;          /* Zf tanh (default: cutoff) */
  double pf_qp, pf_qc, pf_qkf; /* alveliusP, alveliusC, alveliusKf (QfForcing) */
  double les_test_width;       /* dynamic models: TestFilterWidth (<= 0: twice the filter width) */
  double les_cmin;             /* dynamic models: cmin, the smallest coefficient kept */
  double spec_fil;             /* specFil nf (Globals.jl:173-182): with nf != 0 every stats record also
                                  carries the Stats_fil.txt row (quadratic sums weighted by the Gaussian
                                  filter squared, D = 2 pi lx nf / nx) and the spectrum records the
                                  *_fil spectra; 0: off */
  int32_t les_dynp;            /* with FFS_LES_DYNAMIC / FFS_LES_PIOMELLI: the dynamic P tensor term,
                                  1 dynamicSandP, 2 piomelliSandP (les_types.jl:199-330,
                                  les_real_calc.jl:104-106); 0 none */
  int32_t hv_kind;             /* with hyperviscosity: 0 nuh k^2M (HyperViscosity), 1 the spectral barrier
                                  (hyperViscosity spectralBarrier, hyperviscosity_types.jl:32-48; ETD3rdO only) */
  double hv_initk, hv_endk;    /* spectral barrier: initk, endk (<= 0: the reference defaults
                                  cutoff 2 kx_max / 3 and sqrt(3 cutoff) kx_max, simulationtypes.jl:294-297) */
  int32_t rho_hv;              /* densityHyperViscosity (density_stratification_types.jl:137-148): 0 none,
                                  1 rho_hv_nu k^2M, 2 the spectral barrier; the density's ETD3rdO exponent and
                                  the rhohdiss stats column (AB3 adds no term, as in the reference) */
  double rho_hv_nu;            /* densityHyperViscosityCoefficient */
  int32_t rho_hv_m;            /* densityHyperViscosityM, default 2 */
  double rho_hv_initk, rho_hv_endk; /* densityInitk, densityEndk (<= 0: defaults as above) */
  int32_t rho_les;             /* LES of the fourth field (needs les): 0 none, 1 eddy diffusion nu_t grad rho,
                                  2 vorticity diffusion + (c Delta^2 / 2) w x grad rho (densityLesModel,
                                  density_stratification_types.jl:176-185; a passive scalar under lesModel
                                  takes 1, or 2 with scalarLesModel vorticityDiffusion, simulationtypes.jl
                                  :334-346; les_real_calc.jl:116-135) */
  double rho_les_c;            /* densityVorticityCoefficient (0.1) / scalarVorticityCoefficient (1.0) */
  int32_t radix_split;         /* runtime FFT plans: 0 the default radix split of each axis, k = 1, 2 the
                                  k-th alternative split (where the length has one; the autotuner times
                                  them and keeps the fastest per axis) */
} ffs_params;

#define FFS_PF_NONE 0
#define FFS_PF_RF 1  /* RfForcing functor, src/Forcing_methods/forcing.jl:6-114 */
#define FFS_PF_CRF 2 /* CRfForcing, src/Forcing_methods/cforcing.jl:1-97 */
#define FFS_PF_QF 3  /* QfForcing, src/Forcing_methods/qfforcing.jl:1-81 */
#define FFS_PF_NRF 4 /* NRfForcing, src/Forcing_methods/nrforcing.jl:1-138 */
#define FFS_PF_CNRF 5 /* CNRfForcing, src/Forcing_methods/cnrforcing.jl:1-126 */
#define FFS_PF_A 6   /* AForcing (mode by mode; Stats columns hp,vp), src/Forcing_methods/aforcing.jl:1-87 */

#define FFS_LES_SMAGORINSKY 0 /* nu_t = c^2 D^2 |S| (les_real_calc.jl:77-79) */
#define FFS_LES_VREMAN 1      /* VremanLESModel.jl, les_real_calc.jl:132-139 */
#define FFS_LES_PRODUCTION 2  /* ProductionViscosityLESModel.jl */
#define FFS_LES_SILVIS 3      /* silvismodel.jl */
#define FFS_LES_STABLE_NL 4   /* stablenonlinearmodel.jl */
#define FFS_LES_DYNAMIC 5     /* dynamic Smagorinsky: Germano coefficient from a Gaussian test filter,
                                 averaged by the same filter (dynamic_smagorinsky.jl, dynamic_piomelli.jl
                                 :13-26, les_real_calc.jl:71-73); grids with nx <= 512 in FP64 */
#define FFS_LES_PIOMELLI 6    /* piomelliSmagorinsky: the dynamic model with the coefficient of the
                                 previous step extrapolated in time inside the test-filtered stress
                                 (dynamic_smagorinsky.jl:9-19, 172-185, dynamic_piomelli.jl:1-11) */

/* Fill defaults: reference defaults for every key that has one. */
int ffs_params_default(ffs_params* p);

/* Build a simulation (parameters(), src/simulationtypes.jl:242-365). */
int ffs_create(const ffs_params* p, ffs_handle** h);

/* Load physical fields (the reference reads u1.N u2.N u3.N [rho.N],
 * src/simulationtypes.jl:276, src/density_stratification_types.jl:166).
 * rho may be NULL (zero density). layout 0: nx*ny*nz, 1: padded 2*(nx/2+1)*ny*nz. */
int ffs_set_fields(ffs_handle* h, const double* u1, const double* u2, const double* u3, const double* rho,
                   int32_t layout);

/* initialize!(s) (src/FluidFlowSimulation.jl:67-91): forward transform, first
 * right-hand side, integrator history. */
int ffs_initialize(ffs_handle* h);

/* advance_in_time!(s) nsteps times (src/models.jl:3-17). Records Stats rows at
 * iterations multiple of dtStat and u spectra at multiples of dtSpec on the device. */
int ffs_step(ffs_handle* h, int64_t nsteps);

/* The tail of run_simulation after its time loop (src/FluidFlowSimulation.jl:46-49):
 * calculate_rhs!(s) (set_dt! included), the forcing, and writestats(s) at the current
 * iteration. Records one Stats row whatever the iteration (its non-linear and pressure
 * columns are those of the last stats iteration unless this is one, as the reference's
 * s.nlstats/s.pressstats are) and, at a multiple of dtSpec, a spectrum record. Fields,
 * iteration and time do not change. Meant as the run's last call, as in the reference. */
int ffs_finalize(ffs_handle* h);

/* State of the kz = 0 plane forcing, per 2D shell (compute_shells2D, src/utils.jl:161-182).
 * ffs_forcing_shells: the shell count (0 without plane forcing). ffs_forcing_array moves
 * one per-shell array to (set 0) or from (set 1) the host: which 0 = R, the ODE state of
 * rfForcing/cRfForcing (the reference's R.N files, forcing_types.jl:70-72,
 * FluidFlowSimulation.jl:60-62); 1 = Em, the target spectrum (from the initial field at
 * ffs_initialize, or set from targSpectrum.dat after it, forcing_types.jl:76-83);
 * 2 = the shells' mean wavenumber avgK (read only); 3 = N, the plane's non-linear transfer
 * spectrum of nRfForcing/cNRfForcing (the N.N files, forcing_types.jl:114-116); 4 = Ef, the
 * shell energy of the last forcing call (read only; the Eh.N files, output.jl:45-67). n must
 * equal the shell count. aForcing keeps its state per mode and has no shells: which 5 moves
 * its R as the reference's (nx/2+1) x ny matrix in Julia's vec order (kx fastest), n =
 * (nx/2+1)*ny (forcing_types.jl:87-118; its R.N files). */
int ffs_forcing_shells(const ffs_handle* h);
int ffs_forcing_array(ffs_handle* h, int32_t which, double* v, int32_t n, int32_t set);

/* The LES fields of writeoutput (src/output.jl:22-42): the stress T11 T12 T13 T22 T23, the
 * dynamic models' coefficient cs (and cp with the dynamic P tensor), and with the density's
 * LES the flux dflux1..3 (its LES part, nu_t grad rho (+ the vorticity term)). They exist
 * only during a step's calculate_rhs!, so they are captured there: after
 * ffs_capture_output(h, 1) every step that starts at a multiple of write_time, except the
 * first after ffs_initialize (is_output_time, src/simulationtypes.jl:102), and the
 * run's tail (ffs_finalize) store them into a device buffer of nx*ny*nz doubles per field
 * (allocated by the first call that switches it on; a no-op without an LES model);
 * ffs_capture_output(h, 0) stops the capture and keeps the buffer. ffs_output_field copies one
 * field of the most recent capture ([z][y][x], x fastest) and its iteration; FFS_EINVAL
 * for a field this configuration does not have, FFS_ESTATE before the first capture.
 * Capture steps run the generic x pass (not the FP32 register-fused one), so an FP32
 * run with capture differs from one without at FP32 rounding; FP64 runs do not. */
#define FFS_OUT_T11 0
#define FFS_OUT_T12 1
#define FFS_OUT_T13 2
#define FFS_OUT_T22 3
#define FFS_OUT_T23 4
#define FFS_OUT_CS 5
#define FFS_OUT_CP 6
#define FFS_OUT_DFLUX1 7
#define FFS_OUT_DFLUX2 8
#define FFS_OUT_DFLUX3 9
int ffs_capture_output(ffs_handle* h, int32_t on);
int ffs_output_field(ffs_handle* h, int32_t field, double* out, int64_t* iteration);

/* Physical fields at the current iteration (real!(s.u), src/output.jl:1-8). */
int ffs_get_fields(ffs_handle* h, double* u1, double* u2, double* u3, double* rho, int32_t layout);

/* Spectral state as the reference's s.u.c: complex128 half spectrum [nz][ny][nx/2+1]
 * (interleaved re,im; zero outside the retained box). comp: 0..2 velocity, 3 density. */
int ffs_get_spectral(ffs_handle* h, int32_t comp, double* out);
int ffs_set_spectral(ffs_handle* h, int32_t comp, const double* in);

/* Stats.txt header (statsheader, src/stats.jl:1-7) and number of columns per row. */
int ffs_stats_header(const ffs_handle* h, char* buf, int64_t len);
int32_t ffs_stats_ncols(const ffs_handle* h);
/* Columns kept per record: the Stats.txt columns, then 9 integral-length plane sums
 * and 4 derivative variances (inputs of Scales.txt, src/stats.jl:74-109). */
int32_t ffs_record_ncols(const ffs_handle* h);
/* Move up to max_rows pending stats records to the host (oldest first). */
int64_t ffs_stats_records(ffs_handle* h, double* out, int64_t max_rows);

/* Spectra of write_spec (src/spec.jl:1-146,196-450) at iterations multiple of dtSpec:
 * every field binned by calculate_specHV into an H spectrum (lenH) and a V spectrum
 * (lenV). ffs_spectrum_fields gives the field names, comma-separated, in record order
 * (u_h, u_v, vis_h, vis_v, nl_h, nl_v, press_h, press_v, then les_h, les_v with LES,
 * hvis_h, hvis_v with hyperviscosity, buoyancy_v, rho, rhodiss, rhonl with density) and
 * returns their count F. A record is [iteration, then per field: specH(lenH), specV(lenV)],
 * 1 + F (lenH + lenV) doubles. */
/* The Stats.txt row of the most recent stats iteration (writestats, stats.jl:1-62;
 * ffs_stats_ncols columns), without consuming ffs_stats_records. FFS_ESTATE before the
 * first stats iteration. */
int ffs_stats(ffs_handle* h, double* row, int32_t ncols);
/* u spectrum of the current state (spectrum_u + calculate_specHV, spec.jl:316-327,
 * 424-450): specH = the reference's u.specH (total 1/2 |u|^2 on the horizontal bins KH),
 * specV = u_h.specV + u_v.specV (on the vertical bins KRZ). lenH, lenV must equal
 * ffs_spectrum_lengths. */
int ffs_spectrum(ffs_handle* h, double* specH, double* specV, int64_t lenH, int64_t lenV);
int ffs_spectrum_lengths(const ffs_handle* h, int32_t* lenH, int32_t* lenV);
int ffs_spectrum_fields(const ffs_handle* h, char* buf, int64_t len);
int64_t ffs_spectrum_records(ffs_handle* h, double* out, int64_t max_rows);

int64_t ffs_iteration(const ffs_handle* h);
double ffs_time(const ffs_handle* h);
double ffs_dt(const ffs_handle* h);

/* Timing: run nsteps steps and return the elapsed device time (CUDA events on the
 * handle's stream, steps captured in a CUDA graph). */
int ffs_time_steps(ffs_handle* h, int64_t nsteps, double* ms);
/* Per-kernel timing of nsteps steps launched one kernel at a time with CUDA events
 * around each launch. names: comma-separated kernel names; ms: per kernel total. */
int ffs_profile_kernels(ffs_handle* h, int64_t nsteps, char* names, int64_t names_len, double* ms, int32_t max_k,
                        int32_t* nk);
/* Kernel launches per step (for launch counting). */
int32_t ffs_launches_per_step(const ffs_handle* h);
/* Device bytes held by the handle. */
int64_t ffs_device_bytes(const ffs_handle* h);
/* Launch shapes chosen by the autotuner (ffs_params.autotune) with the candidates'
 * timings, as text; empty when autotuning was off. No counterpart in the reference. */
int ffs_tuning_report(const ffs_handle* h, char* buf, int64_t len);
/* The handle's cudaStream_t. */
void* ffs_stream(const ffs_handle* h);

/* No counterpart in the reference. The forward transform of one field (real 3D FFT,
 * 2/3 dealiasing, 1/(nx ny nz) scaling, FP64) for callers that cannot allocate device
 * memory: hosts whose device memory belongs to another allocator or pool (a cudaMalloc
 * of their own would bypass its accounting and fragment it), loops that must not
 * allocate once running (cudaMalloc/cudaFree can synchronise the device and take an
 * unbounded time), plug-in hosts that grant only the buffers they pass in.
 * phys: device pointer, nx*ny*nz doubles, x fastest. spec: device pointer, complex128
 * [nz][ny][nx/2+1] (interleaved re,im), zeros outside the retained modes -- the layout
 * ffs_get_spectral returns. stream: a cudaStream_t (NULL: the legacy default stream);
 * the call only enqueues device work (four kernels and a memset of spec) and reads no
 * host memory from the device. No cudaMalloc/cudaFree: the twiddle tables and the
 * intermediates live in one static device array of 24 MiB per GPU (held until exit), so
 * grids whose intermediates exceed it are rejected with FFS_EINVAL (128^3 with the 2/3
 * rule fits). The first call on a device resolves the array's address
 * (cudaGetSymbolAddress, cached); make that first call before any stream capture.
 * Every call rewrites the twiddles and intermediates in that one array: calls whose
 * work overlaps on the GPU race. Errors: ffs_last_error(NULL). */
int ffs_fourier_noalloc(const double* phys, double* spec, int32_t nx, int32_t ny, int32_t nz, double lx, double ly,
                        double lz, double cutoff, void* stream);

/* No counterpart in the reference. FP64 arithmetic rate of a GPU measured with this
 * library's own register-chain kernels (every SM x 8 CTAs x 256 threads, 8 independent
 * chains per thread): fused multiply-adds (2 flops each) and adds (1 flop each), in
 * TFLOP/s. The denominator of the FP64 plain form's roofline (its transforms are FP64-
 * pipe-bound on GB300). Allocates 8 bytes of device memory for the duration. */
int ffs_measure_fp64_peak(int32_t device, double* fma_tflops, double* add_tflops);

const char* ffs_last_error(const ffs_handle* h);
void ffs_destroy(ffs_handle* h);

/* ---------------------------------------------------------------------------------
 * Batched serving. No counterpart in the reference, which runs one simulation per
 * Julia process through run_simulation() (src/FluidFlowSimulation.jl:23-65); each
 * request here is that run for nt steps with its own `global` parameters and fields.
 *
 * A server owns one GPU stream and a background thread. Requests (FP32 only, grid
 * sides up to max_n, velocity-only or Smagorinsky LES, ETD3 or AB3) queue on submit;
 * the thread admits them while the device memory budget and max_active allow, runs
 * set_fields + initialize! for each on its own stream, and advances every admitted
 * simulation by one step per replay of a single CUDA graph whose kernels walk a work
 * table of (simulation, block) entries. Finished simulations leave the table and their
 * buffers return to a pool for requests of the same grid and model. Each simulation's
 * arithmetic is the same alone and in any mix. Every few replays the thread reads each
 * simulation's error flag; a simulation that produced a non-finite value leaves the
 * batch at once with status FFS_ENAN and frees its slot.
 * Thread safety: every ffs_server entry point may be called from any host thread.
 * --------------------------------------------------------------------------------- */
typedef struct ffs_server ffs_server;

#define FFS_QUEUED 1  /* ffs_result.status: waiting for admission */
#define FFS_RUNNING 2 /* ffs_result.status: in the batch */

typedef struct ffs_server_cfg {
  int32_t device;          /* CUDA device ordinal */
  int64_t memory_budget;   /* device bytes the simulations may hold (admission limit) */
  int32_t max_active;      /* simulations advanced together at most */
  int32_t max_n;           /* largest grid side accepted (<= 128) */
  int32_t autotune;        /* 1: at create, time every kernel form of each size class's passes on
                              probe simulations and keep the fastest per pass (ffs_server_tuning) */
  int32_t class_forms;     /* without autotune: 0 the default forms; 1 every size class's y/z passes one
                              line per thread with 8 kx lines a tile and its x passes generic with 4
                              (y,z) lines; 2 the same with 4 kx lines and 2 (y,z) lines */
} ffs_server_cfg;

typedef struct ffs_request {
  ffs_params params;       /* the simulation's parameters; precision must be FFS_FP32 */
  const double* u1;        /* initial velocity, nx*ny*nz doubles each, x fastest (copied) */
  const double* u2;
  const double* u3;
  int64_t nt;              /* steps after initialize */
  int32_t keep_fields;     /* 1: keep the final physical fields for ffs_fetch_fields */
} ffs_request;

typedef struct ffs_result {
  int32_t status;          /* FFS_OK (finished), FFS_QUEUED, FFS_RUNNING or an FFS_E* code */
  int64_t iteration;       /* final s.iteration */
  double time, dt;         /* final s.time and dt */
  int64_t stats_rows;      /* stats records kept for ffs_fetch_stats */
  int32_t record_ncols;    /* columns per record (as ffs_record_ncols) */
  double submit_s, admit_s, done_s;   /* seconds since ffs_server_create; -1: not yet */
} ffs_result;

typedef struct ffs_server_info {
  int64_t batch_steps;     /* graph replays so far */
  int64_t sim_steps;       /* simulation steps so far (sum over the batch) */
  int32_t active;          /* simulations in the batch now */
  int32_t queued;          /* requests waiting */
  int64_t bytes_in_use;    /* device bytes held by simulations (pool included) */
  int64_t peak_bytes;      /* largest bytes_in_use so far */
  int32_t peak_active;     /* largest batch so far */
} ffs_server_info;

int ffs_server_default(ffs_server_cfg* cfg);
int ffs_server_create(const ffs_server_cfg* cfg, ffs_server** out);
/* Queue a request; *id identifies it in later calls. */
int ffs_submit(ffs_server* s, const ffs_request* r, uint64_t* id);
/* Status of a request without waiting. For a failed request (negative status) the
 * message is in ffs_server_last_error(s). */
int ffs_poll(ffs_server* s, uint64_t id, ffs_result* out);
/* Wait up to timeout_s seconds for a request to finish (FFS_ETIMEDOUT otherwise). */
int ffs_wait(ffs_server* s, uint64_t id, double timeout_s, ffs_result* out);
/* Stats records of a finished request (ffs_stats_records layout); returns rows copied,
 * or the rows available when out is NULL. */
int64_t ffs_fetch_stats(ffs_server* s, uint64_t id, double* out, int64_t max_rows);
/* Final physical fields of a finished request submitted with keep_fields (layout 0). */
int ffs_fetch_fields(ffs_server* s, uint64_t id, double* u1, double* u2, double* u3);
/* Forget a finished request and its results. */
int ffs_release(ffs_server* s, uint64_t id);
/* Cancel a queued or running request: it finishes with status FFS_ECANCELED (a running
 * one before its next batched step; the stats records of the steps it took stay
 * fetchable). FFS_ESTATE when the request has already finished. */
int ffs_cancel(ffs_server* s, uint64_t id);
/* Hold (1) or resume (0) admission: queued requests wait while the batch keeps running. */
int ffs_server_pause(ffs_server* s, int32_t paused);
int ffs_server_stats(ffs_server* s, ffs_server_info* out);
/* The size-class autotuner's report (cfg.autotune): per class, every timed kernel form of
 * each pass and the forms kept. Copies up to len-1 characters; returns the full length. */
int64_t ffs_server_tuning(ffs_server* s, char* buf, int64_t len);
const char* ffs_server_last_error(ffs_server* s);
/* Stop the server (unfinished requests are dropped) and free its GPU memory. */
void ffs_server_destroy(ffs_server* s);

#ifdef __cplusplus
}
#endif
#endif /* FFS_H */
