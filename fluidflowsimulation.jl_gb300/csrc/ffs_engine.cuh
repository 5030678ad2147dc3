// Host side of the engine for one arithmetic type: buffers, launch geometry, the
// CUDA-graph step, set/get of fields and records.
#pragma once
#include <math.h>
#include <string.h>

#include <algorithm>
#include <cstdio>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "ffs_engine.h"
#include "ffs_kernels.cuh"
#include "ffs_pairs.cuh"
#include "ffs_xfused.cuh"
#include "ffs_xles.cuh"
#include "ffs_batch.cuh"
#include "ffs_dynamic.cuh"

namespace ffsgpu {

#define FFS_CK(call)                                                                     \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess) {                                                             \
      err = std::string(#call) + ": " + cudaGetErrorString(e_);                          \
      return FFS_ECUDA;                                                                  \
    }                                                                                    \
  } while (0)

// Radix plans (product == n), radix-3 last. Variant 0 is the default (largest radix
// first, fewest passes); the others are the alternative splits the autotuner times for
// the runtime-plan passes. Returns false for an unsupported n or variant.
inline int plan_variants(int n) {
  switch (n) {
    case 8: return 1;
    case 16: case 32: case 48: case 64: case 96: case 128: case 192: case 256: case 384: case 512: case 768:
    case 1024: return n == 16 || n == 384 || n == 768 ? 2 : 3;
    default: return 0;
  }
}
inline bool make_plan(int n, FftPlan& P, int variant = 0) {
  static const int kRad[][3][4] = {
      // n = 8 .. 1024: up to three splits each, {0} = absent
      {{8}, {0}, {0}},                                              // 8
      {{16}, {4, 4}, {0}},                                          // 16
      {{8, 4}, {4, 8}, {16, 2}},                                    // 32
      {{4, 4, 3}, {16, 3}, {8, 2, 3}},                              // 48
      {{8, 8}, {16, 4}, {4, 16}},                                   // 64
      {{8, 4, 3}, {4, 8, 3}, {16, 2, 3}},                           // 96
      {{16, 8}, {8, 16}, {8, 4, 4}},                                // 128
      {{8, 8, 3}, {16, 4, 3}, {4, 16, 3}},                          // 192
      {{16, 16}, {16, 4, 4}, {8, 8, 4}},                            // 256
      {{16, 8, 3}, {8, 16, 3}, {0}},                                // 384
      {{8, 8, 8}, {16, 8, 4}, {16, 16, 2}},                         // 512
      {{16, 16, 3}, {16, 4, 4, 3}, {0}},                            // 768
      {{16, 8, 8}, {16, 16, 4}, {8, 8, 16}},                        // 1024
  };
  static const int kN[] = {8, 16, 32, 48, 64, 96, 128, 192, 256, 384, 512, 768, 1024};
  int row = -1;
  for (int i = 0; i < 13; ++i)
    if (kN[i] == n) row = i;
  if (row < 0 || variant < 0 || variant >= plan_variants(n)) return false;
  int r[4] = {0, 0, 0, 0}, np = 0, prod = 1;
  for (int i = 0; i < 4 && kRad[row][variant][i]; ++i) { r[i] = kRad[row][variant][i]; prod *= r[i]; ++np; }
  if (prod != n) return false;
  P.n = n; P.np = np;
  int mx = 0, p = 1;
  for (int i = 0; i < 4; ++i) {
    P.r[i] = r[i];
    mx = std::max(mx, r[i]);
    P.T[i] = r[i] ? n / r[i] : 0;
    P.p[i] = p;
    P.tws[i] = r[i] ? n / (p * r[i]) : 0;
    if (r[i]) p *= r[i];
  }
  P.tpl = n / mx;   // threads per line: one butterfly each in the largest-radix pass
  return true;
}

inline int round32(int x) { return ((x + 31) / 32) * 32; }
// real fields into the x pass: u, w [, S] [, the fourth field [, its gradient]]
inline int x_inputs(const ffs_params& p) {
  const bool fld = p.density || p.passive_scalar;
  const bool dl = p.les && fld && (p.rho_les || p.passive_scalar);
  return 6 + (p.les ? 5 : 0) + (fld ? 1 : 0) + (dl ? 3 : 0);
}

template <typename T>
class Engine : public EngineBase {
 public:
  static constexpr int TX = sizeof(T) == 4 ? 8 : 4;   // kx lines per CTA in the y/z passes
  static constexpr int MAXT = 512;   // threads per CTA (launch bounds)
  Inst<T> I;
  ffs_params P;
  cudaStream_t s = nullptr;
  cudaStream_t s2 = nullptr;        // side branch of the step (scalar kernel, ETD table)
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  std::vector<void*> allocs;
  int64_t bytes = 0;
  FieldList inv_list{}, fwd_list{};
  FieldList inv_list_z{};   // the inverse z pass's fields: inv_list without a derived w_z
  // the inverse z pass's fields by prologue family (copy, curl, strain), each launched on
  // its own when split_iz: every CTA of a launch then runs one code path of the kernel
  FieldList inv_fam[3]{};
  int n_fam = 0;
  int split_iz = 0;
  int rad[3] = {0, 0, 0};     // radix-split variant of the x, y, z runtime FFT plans
  int nin = 0, nout = 0;
  int lyz = 4;
  int lio = LYZ_IO;           // (y,z) lines per CTA of the field-IO x kernels
  int xfused = 0;             // n of the register-fused x pass in use (0: generic x pass);
                              // the velocity-only form, or with LES the twelve-field form
  int xfused_ok = 0;          // n for which the fused x pass is available
  bool use_ct = true;         // compile-time FFT plans in the FP32 y/z passes
  bool use_ct_z = true;       // compile-time FFT plans in the FP32 forward z pass
  // form of each compile-time y/z pass: 0 one line per thread, 1 line pairs on the packed
  // FP32 pipe
  int v_iz = 0, v_iy = 0, v_fy = 1;
  bool pair_z = true;         // compile-time one-component forward z pass on line pairs
  bool zseq = false;          // forward z pass: one component at a time (TX lines)
  std::string tune_report;    // candidates and timings of the autotuner
  int txz = TX;               // kx lines per CTA in the forward z pass
  int txy = TX;               // kx lines per CTA in the single-field y/z passes
  int nparts = 0;
  int upd_blocks = 1;
  int n_sms = 1;
  size_t smem_z = 0, smem_y = 0, smem_x = 0, smem_zu = 0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  int n_launch = 0;
  // dynamic Smagorinsky: full-spectrum slots (x-spectral and z-line layouts), the
  // averaged coefficient in physical space, shared memory of its kernels
  DynFull<T> dfull{};
  cplx<T>* dfz = nullptr;
  double* dync = nullptr;
  size_t smem_d0 = 0, smem_d1 = 0, smem_dzf = 0;
  // output capture (writeoutput's LES fields, output.jl:22-42): FP64 planes written by
  // the x pass of each output step, their iteration, the step graph that does it
  double* obuf = nullptr;
  bool out_on = false;        // capture switched on (the buffer stays once allocated)
  int out_nf = 0;
  int64_t out_iter = -1;
  int64_t calls = 0;          // steps since ffs_initialize (the integrator's call counter)
  bool diag_x = false;        // enqueue_step records the capture form of the x pass
  cudaGraph_t graph_out = nullptr;
  cudaGraphExec_t gexec_out = nullptr;

  ~Engine() override {
    if (gexec) cudaGraphExecDestroy(gexec);
    if (graph) cudaGraphDestroy(graph);
    if (gexec_out) cudaGraphExecDestroy(gexec_out);
    if (graph_out) cudaGraphDestroy(graph_out);
    for (void* p : allocs) cudaFree(p);
    if (ev_fork) cudaEventDestroy(ev_fork);
    if (ev_join) cudaEventDestroy(ev_join);
    if (s2) cudaStreamDestroy(s2);
    if (s) cudaStreamDestroy(s);
  }

  template <typename U> int alloc(U** p, size_t count, std::string& err) {
    void* q = nullptr;
    size_t b = count * sizeof(U);
    if (b == 0) b = 16;
    cudaError_t e = cudaMalloc(&q, b);
    if (e != cudaSuccess) {
      err = std::string("cudaMalloc of ") + std::to_string(b) + " bytes: " + cudaGetErrorString(e);
      return e == cudaErrorMemoryAllocation ? FFS_ENOMEM : FFS_ECUDA;
    }
    allocs.push_back(q);
    bytes += (int64_t)b;
    *p = reinterpret_cast<U*>(q);
    FFS_CK(cudaMemsetAsync(q, 0, b, s));
    return 0;
  }

  // retained-range counts for one axis (Globals.jl:132-142, 163-169)
  static void retained(int n, double L, double cutoffr, bool half, int& pos, int& cnt) {
    // k values exactly as rfftfreq / fftfreq compute them
    std::vector<double> k;
    if (half) { for (int i = 0; i <= n / 2; ++i) k.push_back(((double)n / 2 - ((double)n / 2 - i)) / L); }
    else {
      for (int i = 0; i < n / 2; ++i) k.push_back(((double)n / 2 - ((double)n / 2 - i)) / L);
      for (int i = n / 2; i >= 1; --i) k.push_back(-(double)i / L);
    }
    double kmax = 0.0;
    if (half) kmax = k.back();
    else for (double v : k) kmax = std::max(kmax, fabs(v));
    const double c = (cutoffr * kmax) * (cutoffr * kmax);
    pos = 0;
    while (pos < (int)k.size() && !(k[pos] * k[pos] > c) && (half || pos < n / 2)) ++pos;
    if (half) { cnt = pos; return; }
    int neg = 0;
    while (neg < n / 2 && !(k[n - 1 - neg] * k[n - 1 - neg] > c)) ++neg;
    cnt = pos + neg;
  }

  // shared memory of the passes for the current tiles
  void compute_smem() {
    const size_t cb = sizeof(cplx<T>);
    smem_z = (size_t)txy * srows(P.nz) * cb * (I.pz.np >= 3 ? 2 : 1);
    smem_y = (size_t)txy * srows(P.ny) * cb * (I.py.np >= 3 ? 2 : 1);
    if (I.wz_derived) smem_y += sizeof(T) * ((size_t)TX + I.NYR);   // the derived w_z's wavenumber table
    {
      const int PIN = (nin + 1) / 2;
      const int LIN = PIN * lyz;
      const int MXP = I.Mx | 1;
      smem_x = cb * ((size_t)srows(P.nx) * (LIN + 1) +
                     std::max((size_t)nin * lyz * MXP, (size_t)srows(P.nx) * (LIN + 1)));
    }
    smem_zu = cb * ((size_t)zu_lines() * srows(P.nz) * (I.pz.np >= 3 ? 2 : 1) +
                    (size_t)((I.les || I.density) ? 4 : 0) * I.NZR * txz);
    if (I.dyn) {
      smem_d0 = I.dynp ? DynX<0, true>::smem(P.nx, cb) : DynX<0, false>::smem(P.nx, cb);
      smem_d1 = I.dynp ? DynX<1, true>::smem(P.nx, cb) : DynX<1, false>::smem(P.nx, cb);
      smem_dzf = 2 * (size_t)txy * srows(P.nz) * cb;
    }
  }

  // physics parameters (everything that does not change buffer sizes or the step's passes)
  void set_physics(const ffs_params& p) {
    I.nu = p.nu; I.cfl = p.cfl; I.dt0 = p.dt;
    I.ab3 = p.integrator != FFS_ETD3; I.euler = p.integrator == FFS_EULER; I.adaptive = p.variable_dt != 0; I.ref_slot = p.reference_cfl_slot != 0;
    I.hv = p.hyperviscosity != 0; I.hv_m = p.hv_m; I.hv_nu = p.hv_nu;
    {   // the spectral barrier's defaults (simulationtypes.jl:294-297, density_stratification_types.jl
        // :137-141): initk = cutoff 2 kx_max / 3, endk = sqrt(3 cutoff) kx_max, kx_max = (nx/2)/lx
      const double kxm = (double)(p.nx / 2) / p.lx;
      I.hv_kind = p.hv_kind;
      I.hv_initk = p.hv_initk > 0 ? p.hv_initk : p.cutoff * 2 * kxm / 3;
      I.hv_endk = p.hv_endk > 0 ? p.hv_endk : sqrt(p.cutoff * 3) * kxm;
      I.rho_hv = p.density ? p.rho_hv : 0;
      I.rho_hv_nu = p.rho_hv_nu; I.rho_hv_m = p.rho_hv_m;
      I.rho_hv_initk = p.rho_hv_initk > 0 ? p.rho_hv_initk : p.cutoff * 2 * kxm / 3;
      I.rho_hv_endk = p.rho_hv_endk > 0 ? p.rho_hv_endk : sqrt(p.cutoff * 3) * kxm;
    }
    I.les = p.les != 0;
    const double fw = p.filter_width > 0 ? p.filter_width : (p.lx * 2 * M_PI / p.nx) / p.cutoff;
    I.les_alpha = p.smag_c * p.smag_c * fw * fw;
    I.les_model = p.les_model; I.les_c = p.smag_c; I.les_d2 = fw * fw; I.les_cp = p.les_cp; I.les_cb = p.sandp_cb;
    I.dyn = I.les && (p.les_model == FFS_LES_DYNAMIC || p.les_model == FFS_LES_PIOMELLI);
    I.piom = I.les && p.les_model == FFS_LES_PIOMELLI;
    I.dynp = I.dyn ? p.les_dynp : 0;
    {
      const double tw = p.les_test_width > 0 ? p.les_test_width : 2 * fw;   // les_types.jl:390
      I.dyn_d2h = I.dyn ? tw * tw : 0.0;
      I.les_cmin = p.les_cmin;
    }
    I.density = p.density != 0; I.gdir = p.gravity_dir;
    I.scalar = p.passive_scalar != 0;
    // the fourth field's LES diffusion: nu_t grad rho (+ (c D^2 / 2) w x grad rho)
    I.rho_les = (I.les && I.density) ? p.rho_les : 0;
    I.rho_les_c = (p.rho_les_c * I.les_d2) / 2;
    I.alpha = p.density ? p.nu / p.density_pr : 0.0;
    I.dgrad = p.density_gradient; I.gval = p.gravity;
    I.forcing = p.forcing != 0; I.f_eps = p.forcing_power; I.f_kf = p.forcing_kf;
    I.pforce = p.plane_forcing; I.pf_kf = p.pf_kf; I.pf_tf = p.pf_tf; I.pf_alpha = p.pf_alpha; I.pf_cfl = p.cfl;
    I.dt_stat = p.dt_stat; I.dt_spec = p.dt_spec;
    {   // SPEC_FIL_D2 = (2 pi LX nf / NRX)^2 (Globals.jl:173-178)
      const double d = 2 * M_PI * p.lx * p.spec_fil / p.nx;
      I.fil_d2 = d * d;
      I.sfil = I.fil_d2 != 0.0;
    }
    I.Lx_t = (T)p.lx; I.Ly_t = (T)p.ly; I.Lz_t = (T)p.lz;
    I.iLx_t = (T)(1.0 / p.lx); I.iLy_t = (T)(1.0 / p.ly); I.iLz_t = (T)(1.0 / p.lz);
    I.inv_n_t = (T)I.inv_n; I.inv_n2_t = (T)(0.5 * I.inv_n); I.nu_t = (T)p.nu; I.hvnu_t = (T)p.hv_nu; I.alpha_t = (T)I.alpha;
    I.gval_t = (T)p.gravity; I.dgrad_t = (T)p.density_gradient; I.kf2_t = (T)(p.forcing_kf * p.forcing_kf);

  }

  int create(const ffs_params& p_in, std::string& err) override {
    // a passive scalar rides the density's buffers and passes, with g = 0
    // (simulationtypes.jl:198-213): the transport, mean-gradient source and diffusion are
    // the same; buoyancy, the CFL cap, the stats columns and the spectra differ (I.scalar)
    if (p_in.passive_scalar && p_in.density) {
      err = "a passive scalar together with density stratification is not supported";
      return FFS_EUNSUPPORTED;
    }
    if (p_in.rho_les < 0 || p_in.rho_les > 2) { err = "rho_les must be 0, 1 or 2"; return FFS_EINVAL; }
    if (p_in.rho_les && !(p_in.les && (p_in.density || p_in.passive_scalar))) {
      // without an LES model the reference's flux keeps a bare grad rho (nu_t = 1)
      err = "the density / scalar LES diffusion (rho_les) needs an LES model and the density or a passive scalar";
      return FFS_EUNSUPPORTED;
    }
    ffs_params p = p_in;
    // a passive scalar under an LES model always has its LES diffusion, eddy diffusion
    // unless chosen otherwise (simulationtypes.jl:334-346)
    if (p.passive_scalar && p.les && !p.rho_les) p.rho_les = 1;
    if (p.passive_scalar) {
      if (!(p.scalar_pr > 0) || p.scalar_dir < 0 || p.scalar_dir > 2) { err = "bad passive scalar parameters"; return FFS_EINVAL; }
      p.density = 1;
      p.density_pr = p.scalar_pr;
      p.density_gradient = p.scalar_gradient;
      p.gravity = 0.0;
      p.gravity_dir = p.scalar_dir;
    }
    P = p;
    memset(&I, 0, sizeof(I));
    if (p.nx <= 0 || p.ny <= 0 || p.nz <= 0) { err = "grid sizes must be positive"; return FFS_EINVAL; }
    if (!make_plan(p.nx, I.px) || !make_plan(p.ny, I.py) || !make_plan(p.nz, I.pz)) {
      err = "unsupported grid size: each of nx, ny, nz must be one of 8,16,32,48,64,96,128,192,256,384,512,768,1024";
      return FFS_EUNSUPPORTED;
    }
    if (p.radix_split < 0 || p.radix_split > 2) { err = "radix_split must be 0, 1 or 2"; return FFS_EINVAL; }
    {   // an alternative radix split on every axis that has one
      const int ns[3] = {p.nx, p.ny, p.nz};
      FftPlan* pls[3] = {&I.px, &I.py, &I.pz};
      for (int a = 0; a < 3; ++a)
        if (p.radix_split < plan_variants(ns[a])) { make_plan(ns[a], *pls[a], p.radix_split); rad[a] = p.radix_split; }
    }
    if (!(p.lx > 0 && p.ly > 0 && p.lz > 0)) { err = "domain sizes must be positive"; return FFS_EINVAL; }
    if (!(p.cutoff > 0 && p.cutoff <= 1.0)) { err = "cutoff must be in (0, 1]"; return FFS_EINVAL; }
    if (p.dt_stat <= 0 || p.dt_spec <= 0) { err = "dtStat and dtSpec must be positive"; return FFS_EINVAL; }
    if (p.integrator != FFS_ETD3 && p.integrator != FFS_AB3 && p.integrator != FFS_EULER) {
      err = "unknown integrator";
      return FFS_EINVAL;
    }
    if (!p.variable_dt && !(p.dt > 0)) { err = "fixed time stepping needs dt > 0"; return FFS_EINVAL; }
    if (p.hyperviscosity && p.hv_kind == 0 && (p.hv_m < 1 || p.hv_m > 8)) { err = "hyperViscosityM must be in 1..8"; return FFS_EINVAL; }
    if (p.hyperviscosity && (p.hv_kind < 0 || p.hv_kind > 1)) { err = "unknown hyperviscosity kind"; return FFS_EINVAL; }
    if (p.hyperviscosity && p.hv_kind == 1 && p.integrator != FFS_ETD3) {
      // the reference's explicit viscous term needs an exponent M the barrier does not have
      err = "hyperViscosity spectralBarrier needs velocityTimeStep ETD3rdO";
      return FFS_EUNSUPPORTED;
    }
    if (p.rho_hv < 0 || p.rho_hv > 2 || (p.rho_hv == 1 && (p.rho_hv_m < 1 || p.rho_hv_m > 8))) {
      err = "bad densityHyperViscosity";
      return FFS_EINVAL;
    }
    if (p.rho_hv && p.passive_scalar) { err = "densityHyperViscosity takes densityStratification"; return FFS_EINVAL; }
    if (p.density && (p.gravity_dir < 0 || p.gravity_dir > 2)) { err = "gravity direction must be 0..2"; return FFS_EINVAL; }
    if (p.les && (p.les_model < FFS_LES_SMAGORINSKY || p.les_model > FFS_LES_PIOMELLI)) {
      err = "unknown LES model";
      return FFS_EINVAL;
    }
    if (p.plane_forcing) {
      if (p.plane_forcing < FFS_PF_RF || p.plane_forcing > FFS_PF_A) { err = "unknown plane forcing"; return FFS_EINVAL; }
      if (p.integrator == FFS_EULER && (p.plane_forcing == FFS_PF_NRF || p.plane_forcing == FFS_PF_CNRF)) {
        // nrforcing.jl:37 reads the integrator's dt2, which Euller does not keep
        err = "nRfForcing / cNRfForcing need an integrator with a dt history (ETD3rdO or Adams_Bashforth3rdO)";
        return FFS_EUNSUPPORTED;
      }
      if (p.forcing) { err = "isotropicBand and kz = 0 plane forcing together are not supported"; return FFS_EINVAL; }
      if (p.nz < 16) { err = "kz = 0 plane forcing needs nz >= 16 (it forces kz = +-1..+-5)"; return FFS_EUNSUPPORTED; }
      if (p.plane_forcing != FFS_PF_QF && !(p.pf_tf > 0)) { err = "TF must be positive"; return FFS_EINVAL; }
    }
    if (p.les_dynp < 0 || p.les_dynp > 2 ||
        (p.les_dynp && !(p.les && (p.les_model == FFS_LES_DYNAMIC || p.les_model == FFS_LES_PIOMELLI)))) {
      err = "les_dynp (dynamicSandP / piomelliSandP) takes the dynamic Smagorinsky models";
      return FFS_EINVAL;
    }
    if (p.les && p.sandp_cb != 0.0 &&
        ((p.les_model > FFS_LES_PRODUCTION && p.les_model < FFS_LES_DYNAMIC) || p.les_dynp != 0)) {
      err = "SandP takes the Smagorinsky, Vreman, production-viscosity or a dynamic Smagorinsky model";
      return FFS_EINVAL;
    }
    FFS_CK(cudaSetDevice(p.device));
    FFS_CK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    FFS_CK(cudaStreamCreateWithFlags(&s2, cudaStreamNonBlocking));
    FFS_CK(cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming));
    FFS_CK(cudaEventCreateWithFlags(&ev_join, cudaEventDisableTiming));

    I.nx = p.nx; I.ny = p.ny; I.nz = p.nz; I.nxh = p.nx / 2 + 1;
    I.lx = p.lx; I.ly = p.ly; I.lz = p.lz;
    I.inv_n = 1.0 / ((double)p.nx * (double)p.ny * (double)p.nz);
    int xp, xc, yp, yc, zp, zc;
    retained(p.nx, p.lx, p.cutoff, true, xp, xc);
    retained(p.ny, p.ly, p.cutoff, false, yp, yc);
    retained(p.nz, p.lz, p.cutoff, false, zp, zc);
    I.Mx = xc; I.KXP = ((xc + 7) / 8) * 8;
    I.ypos = yp; I.NYR = yc; I.zpos = zp; I.NZR = zc;
    {
      // tabulate ETD coefficients by q = i^2 + j^2 + l^2 when k^2 = q / L^2 is exact
      int ex = 0;
      const double mant = frexp(p.lx, &ex);
      I.uniformL = (p.lx == p.ly && p.ly == p.lz && mant == 0.5);
    }
    // tile sizes: threads per CTA = lines * tpl must stay within the launch bounds
    txy = TX;
    while (txy > TX / 2 && txy * std::max(I.py.tpl, I.pz.tpl) > MAXT) txy /= 2;
    if (txy * std::max(I.py.tpl, I.pz.tpl) > MAXT) { err = "grid size too large for this precision"; return FFS_EUNSUPPORTED; }
    {
      const int nin_x = x_inputs(p);
      const int pin = (nin_x + 1) / 2;
      int maxs = 0;
      FFS_CK(cudaDeviceGetAttribute(&maxs, cudaDevAttrMaxSharedMemoryPerBlockOptin, p.device));
      // (y,z) lines per CTA: within the thread budget and the shared-memory limit
      auto xbytes = [&](int ly) {
        const size_t lin1 = (size_t)pin * ly + 1, mxp = (size_t)(xc | 1);
        return sizeof(cplx<T>) * ((size_t)srows(p.nx) * lin1 + std::max((size_t)nin_x * ly * mxp, (size_t)srows(p.nx) * lin1));
      };
      lyz = 4;
      while (lyz > 1 && (pin * lyz * I.px.tpl > MAXT || xbytes(lyz) + 1024 > (size_t)maxs)) lyz /= 2;
      if (pin * lyz * I.px.tpl > MAXT) { err = "nx too large for this precision"; return FFS_EUNSUPPORTED; }
    }
    if (((long long)p.ny * p.nz) % 4 != 0) { err = "ny*nz must be a multiple of 4"; return FFS_EUNSUPPORTED; }
    // (y,z) lines per CTA of the field-IO x kernels: within the thread and shared-memory limits
    {
      int maxs = 0;
      FFS_CK(cudaDeviceGetAttribute(&maxs, cudaDevAttrMaxSharedMemoryPerBlockOptin, p.device));
      lio = LYZ_IO;
      while (lio > 1 && (2 * lio * I.px.tpl > MAXT || io_bytes(lio, p.nx) + 1024 > (size_t)maxs)) lio /= 2;
      if (2 * lio * I.px.tpl > MAXT) { err = "nx too large for this precision"; return FFS_EUNSUPPORTED; }
    }
    // forward z: from nz = 128 on, one component at a time with TX lines (what the
    // autotuner picks on GB300); below, the three components together
    zseq = p.nz >= 128;
    // default forms of the compile-time y/z passes (the autotuner's picks at 256^3);
    // kernel_variant 2 / 3: every one in its line-pair / one-line-per-thread form
    v_iz = 0; v_iy = 0; v_fy = 1;
    pair_z = p.kernel_variant != 3;
    if (p.kernel_variant == 2) v_iz = v_iy = v_fy = 1;
    if (p.kernel_variant == 3) v_iz = v_iy = v_fy = 0;
    if (p.kernel_variant == 4) {   // half tiles: TX/2 kx lines in the y/z passes, one line per thread
      txy = TX / 2;
      v_iz = v_iy = v_fy = 0;
    }
    txz = TX;
    while (txz > 1 && zu_lines() * I.pz.tpl > MAXT) txz /= 2;
    if (zu_lines() * I.pz.tpl > MAXT) { err = "nz too large for this precision"; return FFS_EUNSUPPORTED; }
    if (txz < TX / 4) { err = "nz too large for this precision"; return FFS_EUNSUPPORTED; }

    set_physics(p);

    // field lists
    nin = 0;
    for (int c = F_UX; c <= F_WZ; ++c) { inv_list.code[nin] = c; inv_list.slot[nin] = nin; ++nin; }
    if (I.les) for (int c = F_SXX; c <= F_SYZ; ++c) { inv_list.code[nin] = c; inv_list.slot[nin] = nin; ++nin; }
    int rho_slot = -1;
    if (I.density) { rho_slot = nin; inv_list.code[nin] = F_RHO; inv_list.slot[nin] = nin; ++nin; }
    if (I.rho_les) for (int c = F_GRX; c <= F_GRZ; ++c) { inv_list.code[nin] = c; inv_list.slot[nin] = nin; ++nin; }
    inv_list.n = nin;
    // the dynamic model's test-filtered u^, S^: transformed with the others, read by its
    // own x kernels only (the x pass reads slots 0..nin-1)
    static_assert(sizeof(FieldList::code) / sizeof(int) >= 15 + (F_GWZ - F_GUX + 1), "FieldList too small");
    if (I.dyn)
      for (int c = F_GUX; c <= (I.dynp ? F_GWZ : F_GSYZ); ++c) {
        inv_list.code[inv_list.n] = c;
        inv_list.slot[inv_list.n] = inv_list.n;
        ++inv_list.n;
      }
    // FP64: w_z and the strain's xx, xy, yy (no kz in them) are formed in the inverse y
    // pass (b_inv_y); the z pass skips them
    I.wz_derived = sizeof(T) == 8;
    inv_list_z = FieldList{};
    for (int i = 0; i < inv_list.n; ++i)
      if (!(I.wz_derived && (inv_list.code[i] == F_WZ || inv_list.code[i] == F_SXX || inv_list.code[i] == F_SXY ||
                             inv_list.code[i] == F_SYY))) {
        inv_list_z.code[inv_list_z.n] = inv_list.code[i];
        inv_list_z.slot[inv_list_z.n] = inv_list.slot[i];
        ++inv_list_z.n;
      }
    {
      FieldList fam[3]{};
      for (int i = 0; i < inv_list_z.n; ++i) {
        const int c = inv_list_z.code[i];
        const int f = (c <= F_UZ || c == F_RHO) ? 0 : (c <= F_WZ ? 1 : 2);
        fam[f].code[fam[f].n] = c;
        fam[f].slot[fam[f].n] = inv_list_z.slot[i];
        ++fam[f].n;
      }
      n_fam = 0;
      for (int f = 0; f < 3; ++f)
        if (fam[f].n) inv_fam[n_fam++] = fam[f];
    }
    split_iz = 0;   // one launch for all families (0.076 ms against 0.097 ms split at 256^3)
    nout = 0;
    auto addo = [&](int role, int slot) { fwd_list.code[nout] = role; fwd_list.slot[nout] = slot; ++nout; };
    addo(R_NX, 0); addo(R_NY, 1); addo(R_NZ, 2); addo(R_KE, 3);
    if (I.les) { addo(R_TXX, 6); addo(R_TXY, 7); addo(R_TXZ, 8); addo(R_TYY, 9); addo(R_TYZ, 10); }
    if (I.density) { addo(R_FX, 4); addo(R_FY, 5); addo(R_FZ, rho_slot); }
    fwd_list.n = nout;
    I.nin = nin; I.nout = nout;
    for (int i = 0; i < nout; ++i) { I.out_role[i] = fwd_list.code[i]; I.out_slot[i] = fwd_list.slot[i]; }
    for (int i = 0; i < nin; ++i) I.in_code[i] = inv_list.code[i];
    const int nslots = std::max(inv_list.n, 4);

    // buffers
    int rc;
    I.ncomp = I.density ? 4 : 3;
    I.cstride = (long long)I.NZR * I.NYR * I.KXP;
    I.fd_kxp = make_fastdiv((unsigned)I.KXP);
    I.fd_nyr = make_fastdiv((unsigned)I.NYR);
    if (I.cstride >= (1ll << 31)) { err = "grid too large (compact spectral component above 2^31 elements)"; return FFS_EUNSUPPORTED; }
    I.wzs = (long long)p.nz * I.NYR * I.KXP;
    I.wys = (long long)p.nz * p.ny * I.KXP;
    cplx<T>* tw[3];
    int ns[3] = {p.nx, p.ny, p.nz};
    for (int a = 0; a < 3; ++a) {
      if ((rc = alloc(&tw[a], ns[a], err))) return rc;
      std::vector<cplx<T>> h(ns[a]);
      for (int t = 0; t < ns[a]; ++t) {
        // exp(-2 pi i t / n) from the FP64 angle, exact at multiples of pi/4
        const double ang = -2.0 * M_PI * (double)t / ns[a];
        double c = cos(ang), sn = sin(ang);
        if ((8 * t) % ns[a] == 0) {
          const int o = (8 * t) / ns[a];
          const double r = sqrt(0.5);
          const double cs8[8] = {1, r, 0, -r, -1, -r, 0, r};
          c = cs8[o]; sn = -cs8[(o + 6) % 8];
        }
        h[t].x = (T)c; h[t].y = (T)sn;
      }
      FFS_CK(cudaMemcpyAsync(tw[a], h.data(), ns[a] * sizeof(cplx<T>), cudaMemcpyHostToDevice, s));
      FFS_CK(cudaStreamSynchronize(s));
    }
    I.twx = tw[0]; I.twy = tw[1]; I.twz = tw[2];
    xfused = 0;
    // the register-fused LES x pass computes the Smagorinsky model only
    const bool smag_only = !p.les || (p.les_model == FFS_LES_SMAGORINSKY && p.sandp_cb == 0.0 && !I.rho_les);
    if (sizeof(T) == 4 && (I.les || !I.density) && p.kernel_variant != 1 && smag_only) {
      int lyzf = 0, rf = 0;
      if (I.les) {   // LES (with or without density): n in {64, 128}
        if (p.nx == 64 || p.nx == 128) { lyzf = XLes<128>::LYZ; rf = XLes<128>::RR; }
      } else {
        switch (p.nx) {
          case 64: lyzf = XFused<64>::LYZ; rf = XFused<64>::R; break;
          case 128: lyzf = XFused<128>::LYZ; rf = XFused<128>::R; break;
          case 256: lyzf = XFused<256>::LYZ; rf = XFused<256>::R; break;
          case 512: lyzf = XFused<512>::LYZ; rf = XFused<512>::R; break;
          case 1024: lyzf = XFused<1024>::LYZ; rf = XFused<1024>::R; break;
          default: break;
        }
      }
      if (lyzf && ((long long)p.ny * p.nz) % lyzf == 0) {
        xfused = xfused_ok = p.nx;
        const int tpl = p.nx / rf;
        // register-pass twiddles [m][i] as (c, c, s, s): both lanes of a packed pair
        cplx<T>* t = nullptr;
        if ((rc = alloc(&t, 2 * (size_t)p.nx, err))) return rc;
        std::vector<cplx<T>> h(2 * (size_t)p.nx), base(p.nx);
        FFS_CK(cudaMemcpyAsync(base.data(), tw[0], p.nx * sizeof(cplx<T>), cudaMemcpyDeviceToHost, s));
        FFS_CK(cudaStreamSynchronize(s));
        for (int m = 0; m < rf; ++m)
          for (int i = 0; i < tpl; ++i) {
            const cplx<T> w = base[(i * m) % p.nx];
            h[2 * (m * tpl + i)] = cplx<T>{w.x, w.x};
            h[2 * (m * tpl + i) + 1] = cplx<T>{w.y, w.y};
          }
        FFS_CK(cudaMemcpyAsync(t, h.data(), 2 * p.nx * sizeof(cplx<T>), cudaMemcpyHostToDevice, s));
        FFS_CK(cudaStreamSynchronize(s));
        I.twx_r = t;
      }
    }
    if ((rc = alloc(&I.uh, (size_t)I.ncomp * I.cstride, err))) return rc;
    if ((rc = alloc(&I.hist, (size_t)2 * I.ncomp * I.cstride, err))) return rc;
    if ((rc = alloc(&I.wz, (size_t)nslots * I.wzs, err))) return rc;
    if ((rc = alloc(&I.wy, (size_t)nslots * I.wys, err))) return rc;
    if ((rc = alloc(&I.st, 1, err))) return rc;
    // CTAs of the stats kernel: at most ~16 modes per thread (per-thread sums stay short)
    nparts = (int)std::max<long long>(1, std::min<long long>((I.cstride + 4095) / 4096, 8192));
    if ((rc = alloc(&I.partials, (size_t)nparts * QPAD, err))) return rc;
    if ((rc = alloc(&I.sbuf, (size_t)((I.les || I.density) ? 8 : 4) * I.cstride, err))) return rc;
    {
      int sms = 0;
      FFS_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, p.device));
      upd_blocks = (int)std::min<long long>((I.cstride + 255) / 256, (long long)sms * 16);
      n_sms = sms;
    }
    // record layout
    ncols_stats = 22 + (I.density ? (I.scalar ? 6 : 8 + (I.rho_les ? 1 : 0) + (I.rho_hv ? 1 : 0)) : 0) + (I.les ? 4 : 0) +
                  (I.pforce == FFS_PF_A ? 2 : ((I.forcing || I.pforce) ? 3 : 0)) + (I.hv ? 3 : 0);
    if (I.pforce && (rc = plane_forcing_tables(p, err))) return rc;
    // a record: the Stats.txt row, 13 Scales.txt inputs, then with specFil the
    // Stats_fil.txt row without iteration and time
    ncols_rec = ncols_stats + 13 + (I.sfil ? ncols_stats - 2 : 0);
    I.ncols = ncols_rec;
    I.rec_cap = p.stats_capacity > 0 ? p.stats_capacity : 256;
    if ((rc = alloc(&I.records, (size_t)I.rec_cap * I.ncols, err))) return rc;
    // spectrum bins (Globals.jl:144-152)
    const double kx1 = 1.0 / p.lx, ky1 = 1.0 / p.ly;
    lenH = kx1 >= ky1 ? p.nx / 2 + 1 : p.ny / 2 + 1;
    I.maxdkh = kx1 >= ky1 ? kx1 : ky1;
    lenV = p.nz / 2 + 1;
    I.dkz = 1.0 / p.lz;
    I.nbinH = lenH; I.nbinV = lenV;
    I.spec_cap = p.spec_capacity > 0 ? p.spec_capacity : 16;
    I.nspecf = SF_BASE_COUNT + (I.les ? 2 : 0) + (I.hv ? 2 : 0) + ((I.density && !I.scalar) ? 4 : 0);
    spec_names = "u_h,u_v,vis_h,vis_v,nl_h,nl_v,press_h,press_v";
    if (I.les) spec_names += ",les_h,les_v";
    if (I.hv) spec_names += ",hvis_h,hvis_v";
    if (I.density && !I.scalar) spec_names += ",buoyancy_v,rho,rhodiss,rhonl";
    if (I.sfil) {   // write_spec's *_fil spectra (spec.jl:17-40, 81-123, 140-143)
      I.nspecf += 8 + (I.hv ? 2 : 0) + ((I.density && !I.scalar) ? 4 : 0);
      spec_names += ",u_fil_h,u_fil_v,vis_fil_h,vis_fil_v,nl_fil_h,nl_fil_v,press_fil_h,press_fil_v";
      if (I.hv) spec_names += ",hvis_fil_h,hvis_fil_v";
      if (I.density && !I.scalar) spec_names += ",buoyancy_fil_v,rho_fil,rhodiss_fil,rhonl_fil";
    }
    if (I.pforce) {   // write_spec_forcing (spec.jl:148-170): the last field of each record
      I.nspecf += 1;
      spec_names += ",forcing_h";
    }
    static_assert(SPEC_MAX_FIELDS >= 31, "spectrum fields");
    nspecf = I.nspecf;
    if ((rc = alloc(&I.spec, (size_t)I.spec_cap * 2 * I.nspecf * std::max(lenH, lenV), err))) return rc;
    // ETD tables
    if (!I.ab3) {
      const long long a = I.Mx - 1, b = std::max(I.ypos - 1, I.NYR - I.ypos), c = std::max(I.zpos - 1, I.NZR - I.zpos);
      I.qmax = (int)(a * a + b * b + c * c);
      const size_t entries = I.uniformL ? (size_t)I.qmax + 1 : (size_t)I.cstride;
      if ((rc = alloc(&I.etab, 4 * entries, err))) return rc;
      if (I.density && (rc = alloc(&I.etab_rho, 4 * entries, err))) return rc;
    }
    // staging for two physical FP64 fields
    if ((rc = alloc(&I.phys, (size_t)2 * p.nx * p.ny * p.nz, err))) return rc;
    if (I.dyn) {
      dfull.kxf = ((I.nxh + 7) / 8) * 8;
      dfull.fys = (long long)p.nz * p.ny * dfull.kxf;
      dfull.gslot0 = nin;
      dfull.nsa = I.dynp ? DYN_NSA_P : DYN_NSA;
      const size_t nsl = I.dynp ? DYN_NSLOTS_P : DYN_NSLOTS, npl = (size_t)p.nx * p.ny * p.nz;
      if ((rc = alloc(&dfull.fy, nsl * dfull.fys, err))) return rc;
      if ((rc = alloc(&dfz, nsl * dfull.fys, err))) return rc;
      // the averaged coefficients in physical space: c [, then cp]
      if ((rc = alloc(&dync, (I.dynp ? 2 : 1) * npl, err))) return rc;
      FFS_CK(cudaMemsetAsync(dync, 0, sizeof(double) * (I.dynp ? 2 : 1) * npl, s));
      I.dyn_c = dync;
      if (I.piom && (rc = alloc(&I.dyn_cm1, npl, err))) return rc;
      if (I.dynp == 2 && (rc = alloc(&I.dyn_cpm1, npl, err))) return rc;
    }

    // launch geometry / shared memory
    compute_smem();
    if ((rc = set_smem(err))) return rc;
    if (p.autotune && (rc = autotune(err))) return rc;

    // state and header
    if ((rc = reset_state(err))) return rc;
    {   // c = cm1 = 0.0289 (les_types.jl:261-266), cp = cpm1 = 0.09 (les_types.jl:298-305)
      const long long np = (long long)p.nx * p.ny * p.nz;
      const unsigned gb = (unsigned)std::min<long long>((np + 255) / 256, 65535);
      if (I.piom) {
        k_dyn_fill<<<gb, 256, 0, s>>>(dync, np, 0.0289);
        k_dyn_fill<<<gb, 256, 0, s>>>(I.dyn_cm1, np, 0.0289);
      }
      if (I.dynp == 2) {
        k_dyn_fill<<<gb, 256, 0, s>>>(dync + np, np, 0.09);
        k_dyn_fill<<<gb, 256, 0, s>>>(I.dyn_cpm1, np, 0.09);
      }
      FFS_CK(cudaGetLastError());
    }
    header = "iteration,time,u1,u2,u3,u1p2,u2p2,u3p2,kh,kv,kaniso,k,dissh,dissv,diss,nlh,nlv,pressh,pressv,tnlh,tnlv,tdiss";
    if (I.scalar) header += ",scalar,scalarp2,dscalardxp2,dscalardyp2,dscalardzp2,scalardiss";
    else if (I.density) header += std::string(",rho,rhop2,drhodxp2,drhodyp2,drhodzp2,rhodiss,trhodiss,bflux") +
                                  (I.rho_les ? ",rhopr" : "") + (I.rho_hv ? ",rhohdiss" : "");
    if (I.les) header += ",prh,prv,praniso,pr";
    if (I.pforce == FFS_PF_A) header += ",hp,vp";
    else if (I.forcing || I.pforce) header += ",hp,vp,tp";
    if (I.hv) header += ",hdissh,hdissv,hdiss";
    FFS_CK(cudaStreamSynchronize(s));
    return 0;
  }

  // The dynamic shared-memory limit is one value per kernel function for the whole
  // process, shared by every engine that launches it: only ever raise it (under a lock),
  // so that an engine of a smaller grid cannot lower it below what a larger one needs.
  template <typename K> int smem_attr(K kern, size_t bytes_, std::string& err) {
    static std::mutex mu;
    std::lock_guard<std::mutex> g(mu);
    cudaFuncAttributes fa;
    FFS_CK(cudaFuncGetAttributes(&fa, kern));
    int maxs = 0;
    FFS_CK(cudaDeviceGetAttribute(&maxs, cudaDevAttrMaxSharedMemoryPerBlockOptin, P.device));
    if (fa.sharedSizeBytes + bytes_ > (size_t)maxs) {
      err = "shared memory per CTA (" + std::to_string(fa.sharedSizeBytes + bytes_) + " bytes) exceeds the device limit";
      return FFS_EUNSUPPORTED;
    }
    if ((int)bytes_ > fa.maxDynamicSharedSizeBytes)
      FFS_CK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes_));
    return 0;
  }

  int set_smem(std::string& err) {
    int dev = P.device, maxs = 0;
    FFS_CK(cudaDeviceGetAttribute(&maxs, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    size_t need[7] = {smem_z, smem_y, smem_x, smem_zu, smem_d0, smem_d1, smem_dzf};
    for (size_t v : need)
      if (v > (size_t)maxs) {
        err = "shared memory per CTA (" + std::to_string(v) + " bytes) exceeds the device limit " + std::to_string(maxs);
        return FFS_EUNSUPPORTED;
      }
    int rc;
    if ((rc = smem_attr(k_inv_z<T, TX>, smem_z, err))) return rc;
    if ((rc = smem_attr(k_inv_y<T, TX>, smem_y, err))) return rc;
    if ((rc = smem_attr(k_fwd_y<T, TX>, smem_y, err))) return rc;
    if ((rc = smem_attr(k_fwd_z_store<T, TX>, smem_z, err))) return rc;
    if ((rc = smem_attr(k_inv_z<T, TX / 2>, smem_z, err))) return rc;
    if ((rc = smem_attr(k_inv_y<T, TX / 2>, smem_y, err))) return rc;
    if ((rc = smem_attr(k_fwd_y<T, TX / 2>, smem_y, err))) return rc;
    if ((rc = smem_attr(k_fwd_z_store<T, TX / 2>, smem_z, err))) return rc;
    if ((rc = smem_attr(xpass_ptr(), smem_x, err))) return rc;
    if (I.dyn && ((rc = smem_attr(I.dynp ? k_dyn_x<T, 0, true> : k_dyn_x<T, 0, false>, smem_d0, err)) ||
                  (rc = smem_attr(I.dynp ? k_dyn_x<T, 1, true> : k_dyn_x<T, 1, false>, smem_d1, err)) ||
                  (rc = smem_attr(k_dyn_zfilter<T, TX>, smem_dzf, err)) ||
                  (rc = smem_attr(k_dyn_zfilter<T, TX / 2>, smem_dzf, err))))
      return rc;
    if constexpr (sizeof(T) == 4) {
      if ((rc = ct_attrs<128>(err)) || (rc = ct_attrs<256>(err)) || (rc = ct_attrs<512>(err)) ||
          (rc = ct_attrs<1024>(err)))
        return rc;
    }
    if constexpr (sizeof(T) == 4) {
      if (I.les) {
        if (xfused == 64 && ((rc = smem_attr(k_x_les<64, false>, XLes<64>::smem(), err)) ||
                             (rc = smem_attr(k_x_les<64, true>, XLes<64>::smem(), err))))
          return rc;
        if (xfused == 128 && ((rc = smem_attr(k_x_les<128, false>, XLes<128>::smem(), err)) ||
                              (rc = smem_attr(k_x_les<128, true>, XLes<128>::smem(), err))))
          return rc;
      } else switch (xfused) {
        case 64: if ((rc = smem_attr(k_x_fused<64>, XFused<64>::smem(), err))) return rc; break;
        case 128: if ((rc = smem_attr(k_x_fused<128>, XFused<128>::smem(), err))) return rc; break;
        case 256: if ((rc = smem_attr(k_x_fused<256>, XFused<256>::smem(), err))) return rc; break;
        case 512: if ((rc = smem_attr(k_x_fused<512>, XFused<512>::smem(), err))) return rc; break;
        case 1024: if ((rc = smem_attr(k_x_fused<1024>, XFused<1024>::smem(), err))) return rc; break;
        default: break;
      }
    }
    if ((rc = smem_attr(zu_ptr(), smem_zu, err))) return rc;
    const size_t io = io_smem();
    if (lio == 4 && ((rc = smem_attr(k_phys_fwd_x<T, 4>, io, err)) || (rc = smem_attr(k_inv_x_phys<T, 4>, io, err)))) return rc;
    if (lio == 2 && ((rc = smem_attr(k_phys_fwd_x<T, 2>, io, err)) || (rc = smem_attr(k_inv_x_phys<T, 2>, io, err)))) return rc;
    if (lio == 1 && ((rc = smem_attr(k_phys_fwd_x<T, 1>, io, err)) || (rc = smem_attr(k_inv_x_phys<T, 1>, io, err)))) return rc;
    return 0;
  }

  // shared-memory limits of the compile-time-length kernels this engine launches
  template <int NC> int ct_attrs(std::string& err) {
    int rc;
    if constexpr (sizeof(T) == 4) {
      constexpr size_t ps = pair_smem<NC, PAIR_LP>();
      const bool full = txy == TX;
      if (full && v_iz == 1 && ctz() == NC && (rc = smem_attr(k_inv_z2<NC, PAIR_LP>, ps, err))) return rc;
      if (full && v_iy == 1 && cty() == NC && (rc = smem_attr(k_inv_y2<NC, PAIR_LP>, ps, err))) return rc;
      if (full && v_fy == 1 && cty() == NC && (rc = smem_attr(k_fwd_y2<NC, PAIR_LP>, ps, err))) return rc;
      if (zpair() && ctzu() == NC && (rc = smem_attr(k_fwd_z2<NC, PAIR_LP>, ps + z2_aux(), err))) return rc;
    }
    if (txy == TX) {
      if (ctz() == NC && (rc = smem_attr(k_inv_z<T, TX, NC>, smem_z, err))) return rc;
      if (cty() == NC && (rc = smem_attr(k_inv_y<T, TX, NC>, smem_y, err))) return rc;
      if (cty() == NC && (rc = smem_attr(k_fwd_y<T, TX, NC>, smem_y, err))) return rc;
    } else if constexpr (NC >= 512) {
      if (ctz() == NC && (rc = smem_attr(k_inv_z<T, TX / 2, NC>, smem_z, err))) return rc;
      if (cty() == NC && (rc = smem_attr(k_inv_y<T, TX / 2, NC>, smem_y, err))) return rc;
      if (cty() == NC && (rc = smem_attr(k_fwd_y<T, TX / 2, NC>, smem_y, err))) return rc;
    }
    if (ctzu() == NC) {
      if (zseq) { if ((rc = smem_attr(k_fwd_z<T, TX, NC, true>, smem_zu, err))) return rc; }
      else if (NC <= 256) { if ((rc = smem_attr(k_fwd_z<T, TX, NC>, smem_zu, err))) return rc; }
      else if ((rc = smem_attr(k_fwd_z<T, 2, NC>, smem_zu, err))) return rc;
    }
    return 0;
  }

  static size_t io_bytes(int l, int nx) { return sizeof(cplx<T>) * (size_t)srows(nx) * 2 * (2 * l + 1); }
  size_t io_smem() const { return io_bytes(lio, P.nx); }
  template <int LIO> void phys_fwd_x(int cnt, int f0) {
    k_phys_fwd_x<T, LIO><<<P.ny * P.nz / LIO, blk(2 * LIO, I.px), io_smem(), s>>>(I, cnt, f0);
  }
  template <int LIO> void inv_x_phys(const Inst<T>& J, int cnt) {
    k_inv_x_phys<T, LIO><<<P.ny * P.nz / LIO, blk(2 * LIO, I.px), io_smem(), s>>>(J, cnt);
  }

  using XK = void (*)(Inst<T>);
  template <int LY> static XK xsel(bool L, bool D, bool DL) {
    if (L && DL) return k_x_pass<T, true, 2, LY>;
    if (L && D) return k_x_pass<T, true, 1, LY>;
    if (L) return k_x_pass<T, true, 0, LY>;
    if (D) return k_x_pass<T, false, 1, LY>;
    return k_x_pass<T, false, 0, LY>;
  }
  XK xpass_ptr() const {
    const bool dl = I.rho_les != 0;
    if (lyz == 4) return xsel<4>(I.les, I.density, dl);
    if (lyz == 2) return xsel<2>(I.les, I.density, dl);
    return xsel<1>(I.les, I.density, dl);
  }
  using ZK = void (*)(Inst<T>, FieldList, int);
  ZK zu_ptr() const {
    if (zseq) return txz == TX ? k_fwd_z<T, TX, 0, true> : k_fwd_z<T, TX / 2, 0, true>;
    if (txz == TX) return k_fwd_z<T, TX>;
    if (txz == TX / 2) return k_fwd_z<T, TX / 2>;
    return k_fwd_z<T, (TX / 4 > 0 ? TX / 4 : 1)>;
  }
  int zu_lines() const { return (zseq ? 1 : 3) * txz; }

  int reset_state(std::string& err) {
    DevState h;
    memset(&h, 0, sizeof(h));
    h.iteration = P.start;
    h.time = P.start_time;
    h.dt = h.dt2 = h.dt3 = P.dt;
    h.nl_h = h.nl_v = h.press_h = h.press_v = 1.0;   // simulationtypes.jl:94-95
    h.nl_hf = h.nl_vf = h.press_hf = h.press_vf = 1.0;
    FFS_CK(cudaMemcpyAsync(I.st, &h, sizeof(h), cudaMemcpyHostToDevice, s));
    FFS_CK(cudaStreamSynchronize(s));
    iteration = h.iteration; time = h.time; dt = h.dt;
    return 0;
  }

  // ---------------------------------------------------------------- launches
  dim3 blk(int lines, const FftPlan& pl) const { return dim3(round32(lines * pl.tpl)); }

  // compile-time FFT lengths of the FP32 y/z passes (0: runtime plan)
  int ct_len(int n) const {
    return (sizeof(T) == 4 && P.kernel_variant != 1 && use_ct && (n == 128 || n == 256 || n == 512 || n == 1024)) ? n : 0;
  }
  // compile-time y/z kernels: TX lines a CTA at every compile-time length, TX/2 lines at
  // 512 and 1024 (where one TX-line CTA takes most of an SM's shared memory)
  int ct_tile(int n) const { return (txy == TX || (txy == TX / 2 && n >= 512)) ? n : 0; }
  int cty() const { return ct_tile(ct_len(I.ny)); }
  static const char* vname_of(int v) { return v == 1 ? "pair" : "1"; }
  int ctz() const { return ct_tile(ct_len(I.nz)); }
  // compile-time forward z kernels exist for TX lines (3 components together or one at a
  // time) at 128/256, and for 2 lines (3 together) or TX lines (one at a time) at 512/1024
  int ctzu() const {
    const int n = use_ct_z ? ct_len_raw(I.nz) : 0;
    if (!n) return 0;
    if (n <= 256) return txz == TX ? n : 0;
    return ((txz == 2 && !zseq) || (txz == TX && zseq)) ? n : 0;
  }

#define FFS_CT_SWITCH(NSEL, CALL)                                    \
  switch (NSEL) {                                                    \
    case 128: { constexpr int NC = 128; CALL; } return;              \
    case 256: { constexpr int NC = 256; CALL; } return;              \
    case 512: { constexpr int NC = 512; CALL; } return;              \
    case 1024: { constexpr int NC = 1024; CALL; } return;            \
    default: break;                                                  \
  }
#define FFS_CT_SWITCH_HALF(NSEL, CALL)                               \
  switch (NSEL) {                                                    \
    case 512: { constexpr int NC = 512; CALL; } return;              \
    case 1024: { constexpr int NC = 1024; CALL; } return;            \
    default: break;                                                  \
  }

  // the paired one-field-at-a-time forward z pass applies (FP32, TX lines, ct plan)
  bool zpair() const { return sizeof(T) == 4 && pair_z && zseq && txz == TX; }
  // its shared accumulators of i k.tau and i k.flux (LES / density)
  size_t z2_aux() const { return (I.les || I.density) ? fwd_z2_aux_bytes<TX>(I.NZR) : 0; }

  // the paired inverse z pass knows the velocity, vorticity, strain and density codes only
  bool pair_codes() const { return !I.dyn && !I.rho_les; }
  void launch_inv_z(const FieldList& F) {
    if constexpr (sizeof(T) == 4) {
      if (txy == TX) {
        if (v_iz == 1 && pair_codes())
          FFS_CT_SWITCH(ctz(), (k_inv_z2<NC, PAIR_LP><<<dim3(F.n, I.KXP / TX, I.NYR), PAIR_LP * ct_tpl<NC>(),
                                                       pair_smem<NC, PAIR_LP>(), s>>>(I, F)))
        FFS_CT_SWITCH(ctz(), (k_inv_z<T, TX, NC><<<dim3(F.n, I.KXP / TX, I.NYR), TX * ct_tpl<NC>(), smem_z, s>>>(I, F)))
      } else {
        FFS_CT_SWITCH_HALF(ctz(), (k_inv_z<T, TX / 2, NC><<<dim3(F.n, I.KXP / (TX / 2), I.NYR), (TX / 2) * ct_tpl<NC>(),
                                                          smem_z, s>>>(I, F)))
      }
    }
    if (txy == TX) k_inv_z<T, TX><<<dim3(F.n, I.KXP / TX, I.NYR), blk(TX, I.pz), smem_z, s>>>(I, F);
    else k_inv_z<T, TX / 2><<<dim3(F.n, I.KXP / (TX / 2), I.NYR), blk(TX / 2, I.pz), smem_z, s>>>(I, F);
  }
  void launch_inv_y(const FieldList& F) {
    if constexpr (sizeof(T) == 4) {
      if (txy == TX) {
        if (v_iy == 1)
          FFS_CT_SWITCH(cty(), (k_inv_y2<NC, PAIR_LP><<<dim3(F.n, I.KXP / TX, I.nz), PAIR_LP * ct_tpl<NC>(),
                                                       pair_smem<NC, PAIR_LP>(), s>>>(I, F)))
        FFS_CT_SWITCH(cty(), (k_inv_y<T, TX, NC><<<dim3(F.n, I.KXP / TX, I.nz), TX * ct_tpl<NC>(), smem_y, s>>>(I, F)))
      } else {
        FFS_CT_SWITCH_HALF(cty(), (k_inv_y<T, TX / 2, NC><<<dim3(F.n, I.KXP / (TX / 2), I.nz), (TX / 2) * ct_tpl<NC>(),
                                                          smem_y, s>>>(I, F)))
      }
    }
    if (txy == TX) k_inv_y<T, TX><<<dim3(F.n, I.KXP / TX, I.nz), blk(TX, I.py), smem_y, s>>>(I, F);
    else k_inv_y<T, TX / 2><<<dim3(F.n, I.KXP / (TX / 2), I.nz), blk(TX / 2, I.py), smem_y, s>>>(I, F);
  }
  void launch_fwd_y(const FieldList& F) {
    if constexpr (sizeof(T) == 4) {
      if (txy == TX) {
        if (v_fy == 1)
          FFS_CT_SWITCH(cty(), (k_fwd_y2<NC, PAIR_LP><<<dim3(F.n, I.KXP / TX, I.nz), PAIR_LP * ct_tpl<NC>(),
                                                       pair_smem<NC, PAIR_LP>(), s>>>(I, F)))
        FFS_CT_SWITCH(cty(), (k_fwd_y<T, TX, NC><<<dim3(F.n, I.KXP / TX, I.nz), TX * ct_tpl<NC>(), smem_y, s>>>(I, F)))
      } else {
        FFS_CT_SWITCH_HALF(cty(), (k_fwd_y<T, TX / 2, NC><<<dim3(F.n, I.KXP / (TX / 2), I.nz), (TX / 2) * ct_tpl<NC>(),
                                                          smem_y, s>>>(I, F)))
      }
    }
    if (txy == TX) k_fwd_y<T, TX><<<dim3(F.n, I.KXP / TX, I.nz), blk(TX, I.py), smem_y, s>>>(I, F);
    else k_fwd_y<T, TX / 2><<<dim3(F.n, I.KXP / (TX / 2), I.nz), blk(TX / 2, I.py), smem_y, s>>>(I, F);
  }
  void launch_fwd_z_store(const FieldList& F) {
    if (txy == TX) k_fwd_z_store<T, TX><<<dim3(F.n, I.KXP / TX, I.NYR), blk(TX, I.pz), smem_z, s>>>(I, F);
    else k_fwd_z_store<T, TX / 2><<<dim3(F.n, I.KXP / (TX / 2), I.NYR), blk(TX / 2, I.pz), smem_z, s>>>(I, F);
  }
  template <int N> void launch_x_fused() {
    if constexpr (sizeof(T) == 4) {
      if (!I.x_pf_dist) {   // CTAs resident at once on the device
        int nb = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_x_fused<N>, XFused<N>::NT, XFused<N>::smem());
        I.x_pf_dist = std::max(1, nb) * n_sms;
      }
    }
    if constexpr (sizeof(T) == 4)
      k_x_fused<N><<<dim3((unsigned)((long long)I.ny * I.nz / XFused<N>::LYZ)), XFused<N>::NT, XFused<N>::smem(), s>>>(I);
  }
  template <int N> void launch_x_les() {
    if constexpr (sizeof(T) == 4) {
      auto k = I.density ? k_x_les<N, true> : k_x_les<N, false>;
      if (!I.x_pf_dist) {   // CTAs resident at once on the device
        int nb = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k, XLes<N>::NT, XLes<N>::smem());
        I.x_pf_dist = std::max(1, nb) * n_sms;
      }
      k<<<dim3((unsigned)((long long)I.ny * I.nz / XLes<N>::LYZ)), XLes<N>::NT, XLes<N>::smem(), s>>>(I);
    }
  }
  template <int LY> static XK xdiag_sel(bool DL) {
    return DL ? k_x_pass_diag<T, 2, LY> : k_x_pass_diag<T, 1, LY>;
  }
  // the capture form of the LES x pass (every LES configuration; density or not)
  XK xdiag_ptr() const {
    const bool dl = I.rho_les != 0;
    if (!I.density) return lyz == 4 ? k_x_pass_diag<T, 0, 4> : (lyz == 2 ? k_x_pass_diag<T, 0, 2> : k_x_pass_diag<T, 0, 1>);
    if (lyz == 4) return xdiag_sel<4>(dl);
    if (lyz == 2) return xdiag_sel<2>(dl);
    return xdiag_sel<1>(dl);
  }
  void launch_x() {
    if (diag_x) {   // an output step: the generic x pass that also stores the output planes
      Inst<T> J = I;
      J.obuf = obuf;
      const int PIN = (nin + 1) / 2;
      xdiag_ptr()<<<dim3(I.ny * I.nz / lyz), blk(PIN * lyz, I.px), smem_x, s>>>(J);
      return;
    }
    if (xfused && I.les) {
      if (xfused == 64) launch_x_les<64>();
      else launch_x_les<128>();
      return;
    }
    switch (xfused) {
      case 64: launch_x_fused<64>(); return;
      case 128: launch_x_fused<128>(); return;
      case 256: launch_x_fused<256>(); return;
      case 512: launch_x_fused<512>(); return;
      case 1024: launch_x_fused<1024>(); return;
      default: break;
    }
    const int PIN = (nin + 1) / 2;
    xpass_ptr()<<<dim3(I.ny * I.nz / lyz), blk(PIN * lyz, I.px), smem_x, s>>>(I);
  }
  void launch_scalar(int mode) { k_scalar<T><<<1, 256, 0, s>>>(I, mode); }
  bool use_table() const { return !I.ab3; }
  // the table is a few thousand FP64-heavy entries: spread them over every SM
  int table_blocks() const {
    const long long count = I.uniformL ? (long long)I.qmax + 1 : I.cstride;
    return (int)std::min<long long>((long long)n_sms * 8, (count + 63) / 64);
  }
  void launch_table(int mode) {
    if (!use_table()) return;
    k_etd_table<T><<<table_blocks(), 64, 0, s>>>(I, mode);
  }
  void launch_zu(int mode) {
    if constexpr (sizeof(T) == 4) {
      const dim3 g(I.KXP / txz, I.NYR);
      if (zpair())
        FFS_CT_SWITCH(ctzu(), (k_fwd_z2<NC, PAIR_LP><<<g, PAIR_LP * ct_tpl<NC>(), pair_smem<NC, PAIR_LP>() + z2_aux(), s>>>(
                                  I, fwd_list, mode)))
      switch (ctzu()) {
        case 128:
          if (zseq) k_fwd_z<T, TX, 128, true><<<g, TX * ct_tpl<128>(), smem_zu, s>>>(I, fwd_list, mode);
          else k_fwd_z<T, TX, 128><<<g, 3 * TX * ct_tpl<128>(), smem_zu, s>>>(I, fwd_list, mode);
          return;
        case 256:
          if (zseq) k_fwd_z<T, TX, 256, true><<<g, TX * ct_tpl<256>(), smem_zu, s>>>(I, fwd_list, mode);
          else k_fwd_z<T, TX, 256><<<g, 3 * TX * ct_tpl<256>(), smem_zu, s>>>(I, fwd_list, mode);
          return;
        case 512:
          if (zseq) k_fwd_z<T, TX, 512, true><<<g, TX * ct_tpl<512>(), smem_zu, s>>>(I, fwd_list, mode);
          else k_fwd_z<T, 2, 512><<<g, 3 * 2 * ct_tpl<512>(), smem_zu, s>>>(I, fwd_list, mode);
          return;
        case 1024:
          if (zseq) k_fwd_z<T, TX, 1024, true><<<g, TX * ct_tpl<1024>(), smem_zu, s>>>(I, fwd_list, mode);
          else k_fwd_z<T, 2, 1024><<<g, 3 * 2 * ct_tpl<1024>(), smem_zu, s>>>(I, fwd_list, mode);
          return;
        default: break;
      }
    }
    zu_ptr()<<<dim3(I.KXP / txz, I.NYR), blk(zu_lines(), I.pz), smem_zu, s>>>(I, fwd_list, mode);
  }
  void launch_update(int mode) { k_update<T><<<upd_blocks, 256, 0, s>>>(I, mode); }
  void launch_stats(int mode) { k_stats<T><<<nparts, 256, 0, s>>>(I, mode); }
  void launch_fin(int mode) { k_finalize<T><<<1, 1024, 0, s>>>(I, mode, nparts); }

  void launch_inv_z_step() {
    if (split_iz && n_fam > 1) {
      for (int f = 0; f < n_fam; ++f) launch_inv_z(inv_fam[f]);
    } else {
      launch_inv_z(inv_list_z);
    }
  }
  // the full-spectrum instance of the dynamic model's filter passes: every kx, ky, kz kept
  Inst<T> full_inst() const {
    Inst<T> J = I;
    J.Mx = I.nxh; J.KXP = dfull.kxf;
    J.NYR = P.ny; J.ypos = P.ny / 2; J.NZR = P.nz; J.zpos = P.nz / 2;
    J.wy = dfull.fy; J.wz = dfz; J.wys = J.wzs = dfull.fys;
    return J;
  }
  // forward y, the z test filter, inverse y on nf full slots from slot0
  void launch_dyn_filter(const Inst<T>& J, int slot0, int nf) {
    FieldList F{};
    F.n = nf;
    for (int i = 0; i < nf; ++i) { F.code[i] = -1; F.slot[i] = slot0 + i; }
    const int t = txy;
    if (t == TX) {
      k_fwd_y<T, TX><<<dim3(nf, J.KXP / TX, P.nz), blk(TX, I.py), smem_y, s>>>(J, F);
      k_dyn_zfilter<T, TX><<<dim3(nf, J.KXP / TX, P.ny), blk(TX, I.pz), smem_dzf, s>>>(J, slot0);
      k_inv_y<T, TX><<<dim3(nf, J.KXP / TX, P.nz), blk(TX, I.py), smem_y, s>>>(J, F);
    } else {
      k_fwd_y<T, TX / 2><<<dim3(nf, J.KXP / (TX / 2), P.nz), blk(TX / 2, I.py), smem_y, s>>>(J, F);
      k_dyn_zfilter<T, TX / 2><<<dim3(nf, J.KXP / (TX / 2), P.ny), blk(TX / 2, I.pz), smem_dzf, s>>>(J, slot0);
      k_inv_y<T, TX / 2><<<dim3(nf, J.KXP / (TX / 2), P.nz), blk(TX / 2, I.py), smem_y, s>>>(J, F);
    }
  }
  // the dynamic coefficient of this step (realspace_LES_calculation!, les_real_calc.jl:3-11)
  void launch_dynamic() {
    const Inst<T> J = full_inst();
    const unsigned lines = (unsigned)((long long)P.ny * P.nz);
    const int nc = I.dynp ? 2 : 1;   // c [, cp]
    (I.dynp ? k_dyn_x<T, 0, true> : k_dyn_x<T, 0, false>)<<<lines, 256, smem_d0, s>>>(I, dfull);
    launch_dyn_filter(J, 0, dfull.nsa);
    (I.dynp ? k_dyn_x<T, 1, true> : k_dyn_x<T, 1, false>)<<<lines, 256, smem_d1, s>>>(I, dfull);
    launch_dyn_filter(J, dfull.nsa, nc);
    Inst<T> C = J;   // physical c [, cp] from the x-spectral full slots
    C.wy = dfull.fy + (long long)dfull.nsa * dfull.fys;
    C.phys = dync;
    if (lio == 4) inv_x_phys<4>(C, nc);
    else if (lio == 2) inv_x_phys<2>(C, nc);
    else inv_x_phys<1>(C, nc);
  }
  void enqueue_step(int mode) {
    launch_inv_z_step();
    launch_inv_y(inv_list);
    if (I.dyn) launch_dynamic();
    launch_x();
    // dt, the integrator's scalars, the band energy and the ETD table need only the x
    // pass (max |u|) and the spectral state: a side branch that overlaps the forward y
    // and z passes, joined before the stats and the update
    cudaEventRecord(ev_fork, s);
    cudaStreamWaitEvent(s2, ev_fork, 0);
    std::swap(s, s2);
    launch_scalar(mode);
    if (!pf_after_fwd()) launch_plane_forcing(mode);
    launch_table(mode);
    std::swap(s, s2);
    cudaEventRecord(ev_join, s2);
    launch_fwd_y(fwd_list);
    launch_zu(mode);
    cudaStreamWaitEvent(s, ev_join, 0);
    if (pf_after_fwd()) launch_plane_forcing(mode);   // reads the step's right-hand side
    launch_stats(mode);
    if (mode != 2) launch_update(mode);   // the run's tail evaluates the rhs and stats only
    launch_fin(mode);
  }
  int launches_per_step() const override {
    return 9 + (use_table() ? 1 : 0) + (I.pforce ? 1 : 0) + ((split_iz && n_fam > 1) ? n_fam - 1 : 0) +
           (I.dyn ? 9 : 0);
  }
  // nRf / cNRf use the plane's non-linear transfer, so they wait for the forward passes
  bool pf_after_fwd() const { return I.pforce == FFS_PF_NRF || I.pforce == FFS_PF_CNRF; }
  void launch_plane_forcing(int mode) {
    if (I.pforce) k_plane_forcing<T><<<1, 256, 0, s>>>(I, mode);
  }

  // kz = 0 plane forcing: 2D shells (compute_shells2D, utils.jl:161-182), Zf (utils.jl
  // :184-198), the Qf power spectrum (build_Qf_power_spectrum!, forcing_types.jl:303-330),
  // and the retained kz = 0 modes listed by shell, on the host in FP64
  int plane_forcing_tables(const ffs_params& p, std::string& err) {
    const int nxh = p.nx / 2 + 1;
    const int nsh = std::min(nxh, p.ny / 2);
    if (nsh + 1 > FFS_PF_MAXSH) { err = "too many forcing shells"; return FFS_EUNSUPPORTED; }
    auto kxv = [&](int i) { return (double)i / p.lx; };
    auto kyv = [&](int y) { return (double)(y < p.ny / 2 ? y : y - p.ny) / p.ly; };   // fftfreq, Nyquist negative
    const double maxdk = std::max(kxv(1), kyv(1));
    std::vector<double> kh(nsh, 0.0), zf(nsh, 0.0), qr(nsh, 0.0);
    std::vector<long long> cnt(nsh, 0);
    for (int j = 0; j < p.ny; ++j)
      for (int i = 0; i < nxh; ++i) {
        const double kx = kxv(i), ky = kyv(j);
        const double K = sqrt(kx * kx + ky * ky);
        const long long ii = llrint(K / maxdk);
        if (ii >= nsh) break;
        kh[ii] += K;
        cnt[ii] += 1;
      }
    for (int i = 0; i < nsh; ++i) kh[i] /= (double)cnt[i];
    const double kf = p.pf_kf;
    for (int i = 0; i < nsh; ++i)
      zf[i] = p.pf_zf_tanh ? tanh((kf - kh[i]) / (0.25 * kf)) * (((kf - kh[i]) <= 0.0) ? 0.0 : 1.0)
                           : (kh[i] <= kf ? 1.0 : 0.0);
    const bool af = p.plane_forcing == FFS_PF_A;
    if (p.plane_forcing == FFS_PF_QF) {
      double integral = 0.0;
      for (int i = 1; i < nsh; ++i)
        if (kh[i] <= kf) {
          const double q = (kh[i] - p.pf_qkf) / p.pf_qc;
          const double term = exp(-(q * q));
          qr[i] = p.pf_qp * term;
          integral += term;
        }
      for (int i = 0; i < nsh; ++i) qr[i] /= integral;
      if (p.les) {   // lfilter: the LES filter width's Gaussian, squared
        const double fw = p.filter_width > 0 ? p.filter_width : (p.lx * 2 * M_PI / p.nx) / p.cutoff;
        const double d2 = fw * fw;
        for (int i = 1; i < nsh; ++i)
          if (kh[i] <= kf) {
            const double G = exp((-d2 / 24) * (kh[i] * kh[i]));
            qr[i] *= G * G;
          }
      }
    }
    // retained kz = 0 modes: spectrum shell (CSR) and forcing shell
    const int plane = I.NYR * I.KXP;
    std::vector<std::vector<int>> byshell(nsh);
    std::vector<int> nmode(plane, -1);
    std::vector<double> zf2(plane, 0.0);   // aForcing: calculate_Zf(d, kf, kx, ky) per mode
    for (int jc = 0; jc < I.NYR; ++jc) {
      const int y = jc < I.ypos ? jc : p.ny - I.NYR + jc;
      for (int ix = 0; ix < I.Mx; ++ix) {
        const double kx = kxv(ix), ky = kyv(y);
        const int m = jc * I.KXP + ix;
        const long long ns = llrint(sqrt(kx * kx + ky * ky) / maxdk);
        if (ns < nsh) byshell[ns].push_back(m);
        if (af) {   // 0 < |k_h| <= kf with |k_h| = sqrt(muladd(kx, kx, ky^2)) (aforcing.jl)
          const double K = sqrt(std::fma(kx, kx, ky * ky));
          if (K > 0 && K <= kf) nmode[m] = 0;
          const double Kz = sqrt(kx * kx + ky * ky);
          zf2[m] = p.pf_zf_tanh ? tanh((kf - Kz) / (0.25 * kf)) * (((kf - Kz) <= 0.0) ? 0.0 : 1.0)
                                : (Kz <= kf ? 1.0 : 0.0);
        } else {
          const long long nf = llrint(sqrt(std::fma(kx, kx, ky * ky)) / maxdk);
          if (nf >= 1 && nf < nsh && kh[nf] <= kf) nmode[m] = (int)nf;
        }
      }
    }
    std::vector<int> start(nsh + 1, 0), modes;
    for (int n = 0; n < nsh; ++n) {
      start[n] = (int)modes.size();
      modes.insert(modes.end(), byshell[n].begin(), byshell[n].end());
    }
    start[nsh] = (int)modes.size();
    // [9][nsh]: R, Em, factor, avgK, Zf, Qf power spectrum, N, Nm1, Ef; then aForcing's
    // [4][plane]: R, Em, factor, Zf per plane mode
    std::vector<double> d(9 * (size_t)nsh + 4 * (size_t)plane, 0.0);
    for (int i = 0; i < nsh; ++i) { d[3 * nsh + i] = kh[i]; d[4 * nsh + i] = zf[i]; d[5 * nsh + i] = qr[i]; }
    for (int m = 0; m < plane; ++m) d[9 * (size_t)nsh + 3 * (size_t)plane + m] = zf2[m];
    int rc;
    double* dd_ = nullptr;
    int *ds = nullptr, *dm = nullptr, *dn = nullptr;
    cplx<T>* df = nullptr;
    if ((rc = alloc(&dd_, d.size(), err)) || (rc = alloc(&ds, start.size(), err)) ||
        (rc = alloc(&dm, std::max<size_t>(modes.size(), 1), err)) || (rc = alloc(&dn, nmode.size(), err)) ||
        (rc = alloc(&df, 2 * (size_t)plane + 20, err)))
      return rc;
    FFS_CK(cudaMemcpyAsync(dd_, d.data(), sizeof(double) * d.size(), cudaMemcpyHostToDevice, s));
    FFS_CK(cudaMemcpyAsync(ds, start.data(), sizeof(int) * start.size(), cudaMemcpyHostToDevice, s));
    if (!modes.empty()) FFS_CK(cudaMemcpyAsync(dm, modes.data(), sizeof(int) * modes.size(), cudaMemcpyHostToDevice, s));
    FFS_CK(cudaMemcpyAsync(dn, nmode.data(), sizeof(int) * nmode.size(), cudaMemcpyHostToDevice, s));
    FFS_CK(cudaMemsetAsync(df, 0, sizeof(cplx<T>) * (2 * (size_t)plane + 20), s));
    FFS_CK(cudaStreamSynchronize(s));
    I.pf_nsh = nsh; I.pf_maxdk = maxdk;
    I.pf_d = dd_; I.pf_start = ds; I.pf_modes = dm; I.pf_nmode = dn; I.pf_force = df;
    pf_avgk = kh;
    return 0;
  }
  std::vector<double> pf_avgk;
  // aForcing's R as the reference's (nx/2+1) x ny matrix, kx fastest (Julia's vec order;
  // forcing_types.jl:362-368, output.jl:49-51); modes outside the retained plane are 0
  int forcing_modes(double* v, int n, int set, std::string& err) {
    const int nxh = I.nxh, plane = I.NYR * I.KXP;
    if (!v || n != nxh * P.ny) { err = "aForcing R: n must be (nx/2+1) * ny"; return FFS_EINVAL; }
    std::vector<double> h(plane, 0.0);
    double* dev = I.pf_d + 9 * (size_t)I.pf_nsh;
    auto ycol = [&](int jc) { return jc < I.ypos ? jc : P.ny - I.NYR + jc; };
    if (set) {
      for (int jc = 0; jc < I.NYR; ++jc)
        for (int ix = 0; ix < I.Mx; ++ix) h[(size_t)jc * I.KXP + ix] = v[(size_t)ycol(jc) * nxh + ix];
      FFS_CK(cudaMemcpyAsync(dev, h.data(), sizeof(double) * plane, cudaMemcpyHostToDevice, s));
      FFS_CK(cudaStreamSynchronize(s));
      return 0;
    }
    FFS_CK(cudaMemcpyAsync(h.data(), dev, sizeof(double) * plane, cudaMemcpyDeviceToHost, s));
    FFS_CK(cudaStreamSynchronize(s));
    std::fill(v, v + n, 0.0);
    for (int jc = 0; jc < I.NYR; ++jc)
      for (int ix = 0; ix < I.Mx; ++ix) v[(size_t)ycol(jc) * nxh + ix] = h[(size_t)jc * I.KXP + ix];
    return 0;
  }

  int forcing_shells() const override { return (I.pforce && I.pforce != FFS_PF_A) ? I.pf_nsh : 0; }
  int forcing_array(int which, double* v, int n, int set, std::string& err) override {
    if (I.pforce == FFS_PF_A && which == 5) return forcing_modes(v, n, set, err);
    if (!I.pforce || I.pforce == FFS_PF_A) { err = "no per-shell plane forcing in this simulation"; return FFS_ESTATE; }
    if (!v || n != I.pf_nsh || which < 0 || which > 4 || (which == 2 && set) || (which == 4 && set)) {
      err = "forcing array: which must be 0 (R), 1 (Em), 2 (avgK, read only), 3 (N) or 4 (Ef, read only), "
            "n the shell count";
      return FFS_EINVAL;
    }
    if (which == 2) { std::copy(pf_avgk.begin(), pf_avgk.end(), v); return 0; }
    const int row = which == 3 ? 6 : (which == 4 ? 8 : which);
    double* dst = I.pf_d + (size_t)row * I.pf_nsh;
    if (set) FFS_CK(cudaMemcpyAsync(dst, v, sizeof(double) * n, cudaMemcpyHostToDevice, s));
    else FFS_CK(cudaMemcpyAsync(v, dst, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
    FFS_CK(cudaStreamSynchronize(s));
    return 0;
  }

  // ---------------------------------------------------------------- fields
  void repack_in(const double* src, double* dst, int layout) const {
    const long long nx = P.nx, ny = P.ny, nz = P.nz;
    if (layout == 0) { memcpy(dst, src, sizeof(double) * nx * ny * nz); return; }
    const long long rx = 2 * (nx / 2 + 1);
    for (long long r = 0; r < ny * nz; ++r) memcpy(dst + r * nx, src + r * rx, sizeof(double) * nx);
  }
  void repack_out(const double* src, double* dst, int layout) const {
    const long long nx = P.nx, ny = P.ny, nz = P.nz;
    if (layout == 0) { memcpy(dst, src, sizeof(double) * nx * ny * nz); return; }
    const long long rx = 2 * (nx / 2 + 1);
    for (long long r = 0; r < ny * nz; ++r) {
      memcpy(dst + r * rx, src + r * nx, sizeof(double) * nx);
      for (long long i = nx; i < rx; ++i) dst[r * rx + i] = 0.0;
    }
  }

  int set_fields(const double* u1, const double* u2, const double* u3, const double* rho, int layout,
                 std::string& err) override {
    if (!u1 || !u2 || !u3) { err = "velocity pointers must not be NULL"; return FFS_EINVAL; }
    if (layout != 0 && layout != 1) { err = "layout must be 0 or 1"; return FFS_EINVAL; }
    const size_t N = (size_t)P.nx * P.ny * P.nz;
    std::vector<double> tmp(2 * N, 0.0);
    const double* src[4] = {u1, u2, u3, rho};
    const int nf = I.density ? 4 : 3;
    for (int pair = 0; pair < 2; ++pair) {
      const int f0 = 2 * pair;
      const int cnt = std::min(2, nf - f0);
      if (cnt <= 0) break;
      for (int k = 0; k < cnt; ++k) {
        if (src[f0 + k]) repack_in(src[f0 + k], tmp.data() + k * N, layout);
        else std::fill(tmp.begin() + k * N, tmp.begin() + (k + 1) * N, 0.0);
      }
      FFS_CK(cudaMemcpyAsync(I.phys, tmp.data(), sizeof(double) * cnt * N, cudaMemcpyHostToDevice, s));
      if (lio == 4) phys_fwd_x<4>(cnt, f0);
      else if (lio == 2) phys_fwd_x<2>(cnt, f0);
      else phys_fwd_x<1>(cnt, f0);
      FFS_CK(cudaGetLastError());
      FFS_CK(cudaStreamSynchronize(s));
    }
    FieldList F{};
    F.n = nf;
    for (int i = 0; i < nf; ++i) { F.code[i] = i; F.slot[i] = i; }
    launch_fwd_y(F);
    launch_fwd_z_store(F);
    FFS_CK(cudaGetLastError());
    // no fourth field given: exactly zero (ScalarField's zeros, density_stratification_types
    // .jl:166), not the rounding that the packed two-field transform leaks from u3 into it
    if (I.density && !rho) FFS_CK(cudaMemsetAsync(I.uh + 3 * I.cstride, 0, sizeof(cplx<T>) * I.cstride, s));
    int rc;
    if ((rc = reset_state(err))) return rc;
    FFS_CK(cudaMemsetAsync(I.hist, 0, sizeof(cplx<T>) * 2 * I.ncomp * I.cstride, s));
    FFS_CK(cudaStreamSynchronize(s));
    initialized = false;
    rec_host.clear(); spec_host.clear();
    return 0;
  }

  int get_fields(double* u1, double* u2, double* u3, double* rho, int layout, std::string& err) override {
    if (layout != 0 && layout != 1) { err = "layout must be 0 or 1"; return FFS_EINVAL; }
    const size_t N = (size_t)P.nx * P.ny * P.nz;
    double* dst[4] = {u1, u2, u3, rho};
    const int nf = I.density ? 4 : 3;
    FieldList F{};
    F.n = nf;
    const int codes[4] = {F_UX, F_UY, F_UZ, F_RHO};
    for (int i = 0; i < nf; ++i) { F.code[i] = codes[i]; F.slot[i] = i; }
    launch_inv_z(F);
    launch_inv_y(F);
    std::vector<double> tmp(2 * N);
    for (int pair = 0; pair < 2; ++pair) {
      const int f0 = 2 * pair;
      const int cnt = std::min(2, nf - f0);
      if (cnt <= 0) break;
      // shift the wanted slots to 0/1 by offsetting the wy base
      Inst<T> J = I;
      J.wy = I.wy + (long long)f0 * I.wys;
      if (lio == 4) inv_x_phys<4>(J, cnt);
      else if (lio == 2) inv_x_phys<2>(J, cnt);
      else inv_x_phys<1>(J, cnt);
      FFS_CK(cudaGetLastError());
      FFS_CK(cudaMemcpyAsync(tmp.data(), I.phys, sizeof(double) * cnt * N, cudaMemcpyDeviceToHost, s));
      FFS_CK(cudaStreamSynchronize(s));
      for (int k = 0; k < cnt; ++k)
        if (dst[f0 + k]) repack_out(tmp.data() + k * N, dst[f0 + k], layout);
    }
    if (!I.density && rho) {
      const long long rx = layout ? 2 * (P.nx / 2 + 1) : P.nx;
      memset(rho, 0, sizeof(double) * rx * P.ny * P.nz);
    }
    return 0;
  }

  int get_spectral(int comp, double* out, std::string& err) override {
    if (comp < 0 || comp >= I.ncomp) { err = "component out of range"; return FFS_EINVAL; }
    std::vector<cplx<T>> h((size_t)I.cstride);
    FFS_CK(cudaMemcpyAsync(h.data(), I.uh + comp * I.cstride, sizeof(cplx<T>) * I.cstride, cudaMemcpyDeviceToHost, s));
    FFS_CK(cudaStreamSynchronize(s));
    const long long nxh = I.nxh;
    memset(out, 0, sizeof(double) * 2 * nxh * P.ny * P.nz);
    for (int kc = 0; kc < I.NZR; ++kc) {
      const int z = kc < I.zpos ? kc : P.nz - I.NZR + kc;
      for (int jc = 0; jc < I.NYR; ++jc) {
        const int y = jc < I.ypos ? jc : P.ny - I.NYR + jc;
        for (int ix = 0; ix < I.Mx; ++ix) {
          const cplx<T> v = h[((long long)kc * I.NYR + jc) * I.KXP + ix];
          const long long o = ((long long)z * P.ny + y) * nxh + ix;
          out[2 * o] = (double)v.x; out[2 * o + 1] = (double)v.y;
        }
      }
    }
    return 0;
  }

  int spectrum_u(double* H, double* V, std::string& err) override {
    const int stride = std::max(lenH, lenV);
    double* d = nullptr;
    FFS_CK(cudaMalloc(&d, sizeof(double) * 2 * stride));
    cudaError_t e = cudaMemsetAsync(d, 0, sizeof(double) * 2 * stride, s);
    if (e == cudaSuccess) {
      k_spectrum_u<T><<<std::max(1, std::min(n_sms * 4, (int)((I.cstride + 255) / 256))), 256, 0, s>>>(I, d, stride);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(H, d, sizeof(double) * lenH, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(V, d + stride, sizeof(double) * lenV, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(d);
    if (e != cudaSuccess) { err = std::string("spectrum: ") + cudaGetErrorString(e); return FFS_ECUDA; }
    return 0;
  }

  int set_spectral(int comp, const double* in, std::string& err) override {
    if (comp < 0 || comp >= I.ncomp) { err = "component out of range"; return FFS_EINVAL; }
    std::vector<cplx<T>> h((size_t)I.cstride);
    memset(h.data(), 0, sizeof(cplx<T>) * h.size());
    const long long nxh = I.nxh;
    for (int kc = 0; kc < I.NZR; ++kc) {
      const int z = kc < I.zpos ? kc : P.nz - I.NZR + kc;
      for (int jc = 0; jc < I.NYR; ++jc) {
        const int y = jc < I.ypos ? jc : P.ny - I.NYR + jc;
        for (int ix = 0; ix < I.Mx; ++ix) {
          const long long o = ((long long)z * P.ny + y) * nxh + ix;
          cplx<T>& v = h[((long long)kc * I.NYR + jc) * I.KXP + ix];
          v.x = (T)in[2 * o]; v.y = (T)in[2 * o + 1];
        }
      }
    }
    FFS_CK(cudaMemcpyAsync(I.uh + comp * I.cstride, h.data(), sizeof(cplx<T>) * I.cstride, cudaMemcpyHostToDevice, s));
    FFS_CK(cudaStreamSynchronize(s));
    initialized = false;
    return 0;
  }

  // ---------------------------------------------------------------- stepping
  int initialize(std::string& err) override {
    int rc;
    if ((rc = reset_state(err))) return rc;
    enqueue_step(1);
    FFS_CK(cudaGetLastError());
    FFS_CK(cudaStreamSynchronize(s));
    if ((rc = pull_state(err))) return rc;
    initialized = true;
    calls = 0;
    out_iter = -1;
    return 0;
  }

  // The tail of run_simulation (FluidFlowSimulation.jl:46-49): calculate_rhs! (set_dt!
  // included), the forcing, and writestats at the current iteration, without an update.
  int finish(std::string& err) override {
    if (!initialized) { err = "ffs_initialize must be called before ffs_finalize"; return FFS_ESTATE; }
    diag_x = out_on;   // the tail's calculate_rhs! feeds the final writeoutput
    enqueue_step(2);
    diag_x = false;
    if (out_on) out_iter = iteration;
    FFS_CK(cudaGetLastError());
    FFS_CK(cudaStreamSynchronize(s));
    return drain(iteration, iteration, err);
  }

  int capture_graph(bool diag, cudaGraph_t* g, cudaGraphExec_t* x, std::string& err) {
    FFS_CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    diag_x = diag;
    enqueue_step(0);
    diag_x = false;
    cudaError_t e = cudaStreamEndCapture(s, g);
    if (e != cudaSuccess) { err = std::string("graph capture: ") + cudaGetErrorString(e); return FFS_ECUDA; }
    FFS_CK(cudaGraphInstantiate(x, *g, 0));
    return 0;
  }
  int build_graph(std::string& err) {
    int rc;
    if (!gexec) {
      if ((rc = capture_graph(false, &graph, &gexec, err))) return rc;
      n_launch = launches_per_step();
    }
    if (obuf && !gexec_out && (rc = capture_graph(true, &graph_out, &gexec_out, err))) return rc;
    return 0;
  }
  // writeoutput runs inside calculate_rhs! when a step starts at a multiple of writeTime,
  // except the first step after initialize! (is_output_time, simulationtypes.jl:102)
  bool output_step(int64_t it, int64_t call) const {
    return out_on && call != 0 && it % P.write_time == 0;
  }

  int capture_output(int on, std::string& err) override {
    out_on = on && I.les;   // the captured fields are the LES model's
    if (!out_on || obuf) return 0;
    out_nf = 5 + (I.dyn ? 1 : 0) + (I.dynp ? 1 : 0) + ((I.rho_les && !I.scalar) ? 3 : 0);
    int rc;
    if ((rc = alloc(&obuf, (size_t)out_nf * P.nx * P.ny * P.nz, err))) return rc;
    if ((rc = smem_attr(xdiag_ptr(), smem_x, err))) return rc;
    return 0;
  }
  // plane of an output field: 0..4 T11 T12 T13 T22 T23, 5 cs, 6 cp, 7..9 dflux1..3
  int out_plane(int field) const {
    if (field >= 0 && field < 5) return field;
    int pl = 5;
    if (field == FFS_OUT_CS) return I.dyn ? pl : -1;
    if (I.dyn) ++pl;
    if (field == FFS_OUT_CP) return I.dynp ? pl : -1;
    if (I.dynp) ++pl;
    if (field >= FFS_OUT_DFLUX1 && field <= FFS_OUT_DFLUX3) return (I.rho_les && !I.scalar) ? pl + field - FFS_OUT_DFLUX1 : -1;
    return -1;
  }
  int output_field(int field, double* out, int64_t* it, std::string& err) override {
    if (!obuf) { err = "output capture is off (ffs_capture_output)"; return FFS_ESTATE; }
    const int pl = out_plane(field);
    if (pl < 0) { err = "this simulation has no such output field"; return FFS_EINVAL; }
    if (out_iter < 0) { err = "no output step has run since the capture was switched on"; return FFS_ESTATE; }
    const size_t N = (size_t)P.nx * P.ny * P.nz;
    FFS_CK(cudaMemcpyAsync(out, obuf + (size_t)pl * N, sizeof(double) * N, cudaMemcpyDeviceToHost, s));
    FFS_CK(cudaStreamSynchronize(s));
    if (it) *it = out_iter;
    return 0;
  }

  DevState hs{};
  int pull_state(std::string& err) {
    FFS_CK(cudaMemcpyAsync(&hs, I.st, sizeof(DevState), cudaMemcpyDeviceToHost, s));
    FFS_CK(cudaStreamSynchronize(s));
    iteration = hs.iteration; time = hs.time; dt = hs.dt;
    return 0;
  }

  // move device records to the host vectors
  int drain(int64_t it_first, int64_t it_last, std::string& err) {
    int rc;
    if ((rc = pull_state(err))) return rc;
    const long long nrec = std::min<long long>(hs.nrec, I.rec_cap);
    if (hs.nrec > I.rec_cap) { err = "stats record buffer overflow"; return FFS_ESTATE; }
    if (nrec > 0) {
      const size_t off = rec_host.size();
      rec_host.resize(off + (size_t)nrec * I.ncols);
      FFS_CK(cudaMemcpyAsync(rec_host.data() + off, I.records, sizeof(double) * nrec * I.ncols, cudaMemcpyDeviceToHost, s));
      FFS_CK(cudaStreamSynchronize(s));
      last_rec.assign(rec_host.end() - I.ncols, rec_host.end());
    }
    const long long nsp = std::min<long long>(hs.nspec, I.spec_cap);
    const int stride = std::max(lenH, lenV);
    if (nsp > 0) {
      const int nq = 2 * I.nspecf;
      std::vector<double> tmp((size_t)nsp * nq * stride);
      FFS_CK(cudaMemcpyAsync(tmp.data(), I.spec, sizeof(double) * tmp.size(), cudaMemcpyDeviceToHost, s));
      FFS_CK(cudaStreamSynchronize(s));
      // iterations of the spectrum records in this chunk
      std::vector<int64_t> its;
      for (int64_t it = it_first; it <= it_last; ++it)
        if (it % P.dt_spec == 0) its.push_back(it);
      for (long long r = 0; r < nsp; ++r) {
        spec_host.push_back(r < (long long)its.size() ? (double)its[r] : -1.0);
        const double* rec = tmp.data() + r * nq * stride;
        for (int q = 0; q < nq; ++q) {
          const int len = (q % 2 == 0) ? lenH : lenV;
          spec_host.insert(spec_host.end(), rec + q * stride, rec + q * stride + len);
        }
      }
      FFS_CK(cudaMemsetAsync(I.spec, 0, sizeof(double) * tmp.size(), s));
    }
    // reset the device counters
    const long long zero = 0;
    FFS_CK(cudaMemcpyAsync(&I.st->nrec, &zero, sizeof(zero), cudaMemcpyHostToDevice, s));
    FFS_CK(cudaMemcpyAsync(&I.st->nspec, &zero, sizeof(zero), cudaMemcpyHostToDevice, s));
    FFS_CK(cudaStreamSynchronize(s));
    if (hs.err & 1u) { err = "non-finite value in the spectral state (simulation diverged)"; return FFS_ENAN; }
    return 0;
  }

  int step(int64_t n, std::string& err) override {
    if (!initialized) { err = "ffs_initialize must be called before ffs_step"; return FFS_ESTATE; }
    if (n < 0) { err = "nsteps must be >= 0"; return FFS_EINVAL; }
    int rc;
    if ((rc = build_graph(err))) return rc;
    int64_t done = 0;
    while (done < n) {
      // chunk so that the device record buffers cannot overflow
      int64_t chunk = 0, ns = 0, nsp = 0;
      const int64_t it0 = iteration + done;
      while (done + chunk < n) {
        const int64_t it = it0 + chunk;
        const int64_t a = (it % P.dt_stat == 0) ? 1 : 0, b = (it % P.dt_spec == 0) ? 1 : 0;
        if (ns + a > I.rec_cap || nsp + b > I.spec_cap) break;
        ns += a; nsp += b; ++chunk;
        if (chunk >= 4096) break;
      }
      for (int64_t i = 0; i < chunk; ++i) {
        const bool o = output_step(it0 + i, calls);
        FFS_CK(cudaGraphLaunch(o ? gexec_out : gexec, s));
        if (o) out_iter = it0 + i;
        ++calls;
      }
      FFS_CK(cudaStreamSynchronize(s));
      if ((rc = drain(it0, it0 + chunk - 1, err))) return rc;
      done += chunk;
    }
    return 0;
  }

  int time_steps(int64_t n, double* ms, std::string& err) override {
    if (!initialized) { err = "ffs_initialize must be called first"; return FFS_ESTATE; }
    int rc;
    if ((rc = build_graph(err))) return rc;
    cudaEvent_t a, b;
    FFS_CK(cudaEventCreate(&a));
    FFS_CK(cudaEventCreate(&b));
    FFS_CK(cudaEventRecord(a, s));
    for (int64_t i = 0; i < n; ++i) FFS_CK(cudaGraphLaunch(gexec, s));
    calls += n;
    FFS_CK(cudaEventRecord(b, s));
    FFS_CK(cudaEventSynchronize(b));
    float f = 0.f;
    FFS_CK(cudaEventElapsedTime(&f, a, b));
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    *ms = f;
    return drain(iteration, iteration + n - 1, err);
  }

  int profile(int64_t n, std::vector<KernelTiming>& out, std::string& err) override {
    if (!initialized) { err = "ffs_initialize must be called first"; return FFS_ESTATE; }
    const char* names[10] = {"inv_z", "inv_y", "x_pass", "fwd_y", "scalar", "etd_table", "fwd_z", "stats",
                             "update", "finalize"};
    double acc[10] = {0};
    cudaEvent_t ev[11];
    for (auto& e : ev) FFS_CK(cudaEventCreate(&e));
    const int64_t it0 = iteration;
    for (int64_t i = 0; i < n; ++i) {
      FFS_CK(cudaEventRecord(ev[0], s));
      launch_inv_z_step(); FFS_CK(cudaEventRecord(ev[1], s));
      launch_inv_y(inv_list); FFS_CK(cudaEventRecord(ev[2], s));
      launch_x(); FFS_CK(cudaEventRecord(ev[3], s));
      launch_fwd_y(fwd_list); FFS_CK(cudaEventRecord(ev[4], s));
      launch_scalar(0);
      launch_plane_forcing(0); FFS_CK(cudaEventRecord(ev[5], s));
      launch_table(0); FFS_CK(cudaEventRecord(ev[6], s));
      launch_zu(0); FFS_CK(cudaEventRecord(ev[7], s));
      launch_stats(0); FFS_CK(cudaEventRecord(ev[8], s));
      launch_update(0); FFS_CK(cudaEventRecord(ev[9], s));
      launch_fin(0); FFS_CK(cudaEventRecord(ev[10], s));
      FFS_CK(cudaEventSynchronize(ev[10]));
      for (int k = 0; k < 10; ++k) {
        float f = 0.f;
        FFS_CK(cudaEventElapsedTime(&f, ev[k], ev[k + 1]));
        acc[k] += f;
      }
    }
    for (auto& e : ev) cudaEventDestroy(e);
    out.clear();
    for (int k = 0; k < 10; ++k) {
      if (k == 5 && !use_table()) continue;
      out.push_back({names[k], acc[k]});
    }
    return drain(it0, it0 + n - 1, err);
  }

  // ---------------------------------------------------------------- autotuning
  // Times the launch shapes each pass can take on this grid, on the engine's own
  // buffers, and keeps the fastest:
  //   y/z passes:  TX or TX/2 lines per CTA, compile-time or runtime FFT plan
  //   x pass:      register-fused (FP32 velocity-only) or generic, 4/2/1 (y,z) lines
  //   forward z:   TX, TX/2 or TX/4 lines; three components together or one at a time
  // Each group is tuned on its own (they are independent passes). The choice is cached
  // per grid, model and precision for the process, so engines of the same shape tune once.
  struct TuneChoice {
    int txy, use_ct, lyz, xfused, txz, zseq, use_ct_z, pair_z, v_iz, v_iy, v_fy, split_iz;
    int rad[3];
    std::string report;
  };
  static std::mutex& tune_mu() { static std::mutex m; return m; }
  static std::map<std::string, TuneChoice>& tune_cache() { static std::map<std::string, TuneChoice> c; return c; }

  int autotune(std::string& err) {
    const std::string key = std::to_string(sizeof(T)) + ":" + std::to_string(P.nx) + "x" + std::to_string(P.ny) + "x" +
                            std::to_string(P.nz) + ":" + std::to_string(I.les) + std::to_string(I.density) +
                            std::to_string(I.dyn) + ":" +
                            std::to_string(I.Mx) + "," + std::to_string(I.NYR) + "," + std::to_string(I.NZR) + ":" +
                            std::to_string(P.kernel_variant);
    {
      std::lock_guard<std::mutex> g(tune_mu());
      auto it = tune_cache().find(key);
      if (it != tune_cache().end()) {
        const TuneChoice& c = it->second;
        txy = c.txy; use_ct = c.use_ct; lyz = c.lyz; xfused = c.xfused; txz = c.txz; zseq = c.zseq;
        use_ct_z = c.use_ct_z; pair_z = c.pair_z; v_iz = c.v_iz; v_iy = c.v_iy; v_fy = c.v_fy;
        split_iz = c.split_iz;
        for (int a = 0; a < 3; ++a) rad[a] = c.rad[a];
        make_plan(P.nx, I.px, rad[0]); make_plan(P.ny, I.py, rad[1]); make_plan(P.nz, I.pz, rad[2]);
        tune_report = c.report + " (cached)";
        compute_smem();
        return set_smem(err);
      }
    }
    int maxs = 0;
    FFS_CK(cudaDeviceGetAttribute(&maxs, cudaDevAttrMaxSharedMemoryPerBlockOptin, P.device));
    const double work = (double)P.nx * P.ny * P.nz;
    const int reps = work > 1.5e8 ? 3 : (work > 2e7 ? 5 : 20);
    cudaEvent_t a, b;
    FFS_CK(cudaEventCreate(&a));
    FFS_CK(cudaEventCreate(&b));
    std::string rep;
    int rc = 0;
    auto timed = [&](auto&& launch, float& ms) -> int {
      compute_smem();
      if (smem_z > (size_t)maxs || smem_y > (size_t)maxs || smem_x > (size_t)maxs || smem_zu > (size_t)maxs) {
        ms = 1e30f;
        return 0;
      }
      int r;
      if ((r = set_smem(err))) return r;
      launch();
      FFS_CK(cudaGetLastError());
      FFS_CK(cudaEventRecord(a, s));
      for (int i = 0; i < reps; ++i) launch();
      FFS_CK(cudaEventRecord(b, s));
      FFS_CK(cudaEventSynchronize(b));
      FFS_CK(cudaGetLastError());
      FFS_CK(cudaEventElapsedTime(&ms, a, b));
      ms /= reps;
      return 0;
    };
    char line[160];
    // y/z passes
    {
      float best = 1e30f;
      int bt = txy, bc = use_ct;
      v_iz = v_iy = v_fy = 0;
      for (int t : {TX, TX / 2})
        for (int c : {1, 0}) {
          if (t * std::max(I.py.tpl, I.pz.tpl) > MAXT) continue;
          const bool half_ct = t == TX / 2 && (ct_len_raw(P.ny) >= 512 || ct_len_raw(P.nz) >= 512);
          if (c && (sizeof(T) != 4 || (t != TX && !half_ct) || (!ct_len_raw(P.ny) && !ct_len_raw(P.nz)))) continue;
          txy = t; use_ct = c;
          float ms = 0.f;
          if ((rc = timed([&] { launch_inv_z(inv_list_z); launch_inv_y(inv_list); launch_fwd_y(fwd_list); }, ms))) break;
          snprintf(line, sizeof(line), "yz[tx=%d,%s]=%.4fms ", t, c ? "ct" : "rt", ms);
          rep += line;
          if (ms < best) { best = ms; bt = t; bc = c; }
        }
      txy = bt; use_ct = bc;
      // then the form of each compile-time pass on its own
      auto pick = [&](int& v, const char* name, int n, auto&& launch) -> int {
        if (!n) return 0;
        float bms = 1e30f;
        int bv = 0;
        for (int c = 0; c < 2; ++c) {
          v = c;
          float ms = 0.f;
          int r;
          if ((r = timed(launch, ms))) return r;
          snprintf(line, sizeof(line), "%s[%s]=%.4fms ", name, vname_of(c), ms);
          rep += line;
          if (ms < bms) { bms = ms; bv = c; }
        }
        v = bv;
        return 0;
      };
      if (!rc) rc = pick(v_iz, "z_inv", (!pair_codes() || txy != TX) ? 0 : ctz(), [&] { launch_inv_z(inv_list_z); });
      // one launch for every field family, or one per family
      if (!rc && n_fam > 1) {
        float bms = 1e30f;
        int bs = 0;
        for (int sp = 0; sp < 2 && !rc; ++sp) {
          split_iz = sp;
          float ms = 0.f;
          rc = timed([&] { launch_inv_z_step(); }, ms);
          snprintf(line, sizeof(line), "z_inv[%s]=%.4fms ", sp ? "split" : "joint", ms);
          rep += line;
          if (ms < bms) { bms = ms; bs = sp; }
        }
        split_iz = bs;
      }
      if (!rc) rc = pick(v_iy, "y_inv", txy == TX ? cty() : 0, [&] { launch_inv_y(inv_list); });
      if (!rc) rc = pick(v_fy, "y_fwd", txy == TX ? cty() : 0, [&] { launch_fwd_y(fwd_list); });
    }
    // x pass
    if (!rc) {
      float best = 1e30f;
      int bl = lyz, bf = xfused;
      const int pin = (nin + 1) / 2;
      std::vector<std::pair<int, int>> cand;   // (fused n, lyz)
      if (xfused_ok) cand.push_back({xfused_ok, lyz});
      for (int l : {4, 2, 1})
        if (pin * l * I.px.tpl <= MAXT) cand.push_back({0, l});
      for (auto& c : cand) {
        xfused = c.first; lyz = c.second;
        float ms = 0.f;
        if ((rc = timed([&] { launch_x(); }, ms))) break;
        snprintf(line, sizeof(line), "x[%s%d]=%.4fms ", c.first ? "fused" : "lyz", c.first ? c.first : c.second, ms);
        rep += line;
        if (ms < best) { best = ms; bl = c.second; bf = c.first; }
      }
      lyz = bl; xfused = bf;
    }
    // forward z pass
    if (!rc) {
      float best = 1e30f;
      int bt = txz, bq = zseq, bc = use_ct_z, bp = pair_z;
      for (int q : {0, 1})
        for (int t : {TX, TX / 2, TX / 4})
          for (int c : {2, 1, 0}) {
            if (t < 1 || (q ? 1 : 3) * t * I.pz.tpl > MAXT) continue;
            if (q && t < TX / 2) continue;
            txz = t; zseq = q; use_ct_z = c > 0; pair_z = c == 2;
            if (c && !ctzu()) continue;   // no compile-time kernel for this shape
            if (c == 2 && !zpair()) continue;
            float ms = 0.f;
            if ((rc = timed([&] { launch_zu(0); }, ms))) break;
            snprintf(line, sizeof(line), "fwd_z[tx=%d,%s,%s]=%.4fms ", t, q ? "seq" : "3c", c == 2 ? "ct2" : c ? "ct" : "rt", ms);
            rep += line;
            if (ms < best) { best = ms; bt = t; bq = q; bc = c > 0; bp = c == 2; }
          }
      txz = bt; zseq = bq; use_ct_z = bc; pair_z = bp;
    }
    // radix splits of the runtime FFT plans, per axis, timed on the passes that run them
    // (every pass in FP64; in FP32 the ones without a compile-time plan)
    if (!rc) {
      const int pin = (nin + 1) / 2;
      const int ns[3] = {P.nx, P.ny, P.nz};
      FftPlan* pls[3] = {&I.px, &I.py, &I.pz};
      const char* an[3] = {"x", "y", "z"};
      for (int ax = 0; ax < 3 && !rc; ++ax) {
        const bool used = ax == 0 ? xfused == 0 : (ax == 1 ? cty() == 0 : (ctz() == 0 || ctzu() == 0));
        const int nv = plan_variants(ns[ax]);
        if (!used || nv < 2) continue;
        const FftPlan keep = *pls[ax];
        float bms = 1e30f;
        int bv = rad[ax];
        for (int v = 0; v < nv && !rc; ++v) {
          FftPlan c;
          if (!make_plan(ns[ax], c, v)) continue;
          // the launch shapes stay within the thread budget with this plan's threads per line
          const int tpl_yz = std::max(ax == 1 ? c.tpl : I.py.tpl, ax == 2 ? c.tpl : I.pz.tpl);
          if (ax == 0 && (pin * lyz * c.tpl > MAXT || 2 * lio * c.tpl > MAXT)) continue;
          if (ax > 0 && (txy * tpl_yz > MAXT || (ax == 2 && zu_lines() * c.tpl > MAXT))) continue;
          *pls[ax] = c;
          float ms = 0.f;
          if (ax == 0) rc = timed([&] { launch_x(); }, ms);
          else if (ax == 1) rc = timed([&] { launch_inv_y(inv_list); launch_fwd_y(fwd_list); }, ms);
          else rc = timed([&] { launch_inv_z_step(); launch_zu(0); }, ms);
          char rs[32];
          int o = 0;
          for (int i = 0; i < c.np; ++i) o += snprintf(rs + o, sizeof(rs) - o, i ? "x%d" : "%d", c.r[i]);
          snprintf(line, sizeof(line), "radix_%s[%s]=%.4fms ", an[ax], rs, ms);
          rep += line;
          if (ms < bms) { bms = ms; bv = v; }
        }
        *pls[ax] = keep;
        rad[ax] = bv;
        make_plan(ns[ax], *pls[ax], bv);
      }
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (rc) return rc;
    snprintf(line, sizeof(line), "-> tx_yz=%d %s [z_inv %s%s, y_inv %s, y_fwd %s], x=%s%d, fwd_z tx=%d %s %s", txy,
             use_ct ? "ct" : "rt", vname_of(v_iz), split_iz ? " split" : "", vname_of(v_iy), vname_of(v_fy),
             xfused ? "fused" : "lyz", xfused ? xfused : lyz, txz, zseq ? "seq" : "3c",
             use_ct_z ? (zpair() ? "ct2" : "ct") : "rt");
    rep += line;
    snprintf(line, sizeof(line), ", radix variants x%d y%d z%d", rad[0], rad[1], rad[2]);
    rep += line;
    tune_report = rep;
    compute_smem();
    if ((rc = set_smem(err))) return rc;
    {
      std::lock_guard<std::mutex> g(tune_mu());
      tune_cache()[key] = TuneChoice{txy, use_ct, lyz, xfused, txz, zseq, use_ct_z, pair_z, v_iz, v_iy, v_fy, split_iz,
                                     {rad[0], rad[1], rad[2]}, rep};
    }
    return reset_state(err);
  }
  int ct_len_raw(int n) const {
    return (sizeof(T) == 4 && P.kernel_variant != 1 && (n == 128 || n == 256 || n == 512 || n == 1024)) ? n : 0;
  }
  std::string tuning() const override { return tune_report; }

  int64_t device_bytes() const override { return bytes; }
  void* stream() const override { return (void*)s; }

  // ---------------------------------------------------------------- batching
  // Device bytes create() allocates for p (the same buffer list, no allocation).
  static int64_t estimate_bytes(const ffs_params& p) {
    FftPlan a, b, c;
    if (!make_plan(p.nx, a) || !make_plan(p.ny, b) || !make_plan(p.nz, c)) return -1;
    int xp, xc, yp, yc, zp, zc;
    retained(p.nx, p.lx, p.cutoff, true, xp, xc);
    retained(p.ny, p.ly, p.cutoff, false, yp, yc);
    retained(p.nz, p.lz, p.cutoff, false, zp, zc);
    const int64_t KXP = ((xc + 7) / 8) * 8, cb = sizeof(cplx<T>);
    const int64_t cs = (int64_t)zc * yc * KXP, wzs = (int64_t)p.nz * yc * KXP, wys = (int64_t)p.nz * p.ny * KXP;
    const int nin = x_inputs(p), nslots = std::max(nin, 4);
    const int ncomp = p.density ? 4 : 3;
    int64_t t = cb * (2 * (int64_t)(2 * p.nx + p.ny + p.nz));   // twiddle tables, packed x table
    t += cb * (3 * ncomp * cs + (int64_t)nslots * (wzs + wys) + ((p.les || p.density) ? 8 : 4) * cs);
    t += 8 * (int64_t)std::min<int64_t>((cs + 4095) / 4096, 8192) * QPAD;
    t += 8 * (int64_t)(p.stats_capacity > 0 ? p.stats_capacity : 256) * 64;   // record columns <= 53
    t += 8 * (int64_t)(p.spec_capacity > 0 ? p.spec_capacity : 16) * 4 * (std::max(p.nx, std::max(p.ny, p.nz)) / 2 + 1);
    if (p.integrator == FFS_ETD3) t += 2 * (int64_t)sizeof(T) * 4 * cs;
    t += 16 * (int64_t)p.nx * p.ny * p.nz;   // FP64 staging of two physical fields
    return t + 4096;
  }

  int batch_export(void* bi, size_t bi_size, BatchGeom* g, std::string& err) const override {
    if (bi_size != sizeof(BatchInst<T>)) { err = "batch parameter block size mismatch"; return FFS_EINVAL; }
    BatchInst<T>* b = reinterpret_cast<BatchInst<T>*>(bi);
    b->I = I;
    b->I.x_pf_dist = 0;   // in a batch the CTA order interleaves simulations: no look-ahead
    b->inv = inv_list;
    b->fwd = fwd_list;
    b->nparts = nparts;
    g->nx = P.nx; g->ny = P.ny; g->nz = P.nz;
    g->nin = inv_list.n; g->nout = fwd_list.n;
    g->kx_tiles = I.KXP / txy;
    g->kxp = I.KXP;
    g->nyr = I.NYR;
    g->yz_groups = P.ny * P.nz / lyz;
    g->fwd_z_tiles = I.KXP / txz;
    g->les = I.les; g->density = I.density; g->etd = !I.ab3;
    g->table_blocks = use_table() ? table_blocks() : 0;
    g->nparts = nparts; g->upd_blocks = upd_blocks;
    g->txy = txy; g->txz = txz; g->lyz = lyz;
    g->xfused = xfused;
    return 0;
  }

  int stream_wait(void* event, std::string& err) override {
    FFS_CK(cudaStreamWaitEvent(s, (cudaEvent_t)event, 0));
    return 0;
  }

  int repurpose(const ffs_params& p, std::string& err) override {
    const bool same = p.nx == P.nx && p.ny == P.ny && p.nz == P.nz && p.lx == P.lx && p.ly == P.ly &&
                      p.lz == P.lz && p.cutoff == P.cutoff && p.integrator == P.integrator &&
                      (p.les != 0) == (P.les != 0) && (p.density != 0) == (P.density != 0) &&
                      (p.forcing != 0) == (P.forcing != 0) && (p.hyperviscosity != 0) == (P.hyperviscosity != 0) &&
                      p.precision == P.precision && p.device == P.device && p.kernel_variant == P.kernel_variant &&
                      (p.stats_capacity > 0 ? p.stats_capacity : 256) <= I.rec_cap &&
                      (p.spec_capacity > 0 ? p.spec_capacity : 16) <= I.spec_cap;
    if (!same) { err = "repurpose needs the same grid, model and record capacities"; return FFS_EINVAL; }
    if (!p.variable_dt && !(p.dt > 0)) { err = "fixed time stepping needs dt > 0"; return FFS_EINVAL; }
    if (p.dt_stat <= 0 || p.dt_spec <= 0) { err = "dtStat and dtSpec must be positive"; return FFS_EINVAL; }
    if (p.hyperviscosity && (p.hv_m < 1 || p.hv_m > 8)) { err = "hyperViscosityM must be in 1..8"; return FFS_EINVAL; }
    const int rc_cap = I.rec_cap, sp_cap = I.spec_cap;
    P = p;
    set_physics(p);
    I.rec_cap = rc_cap; I.spec_cap = sp_cap;
    P.stats_capacity = rc_cap; P.spec_capacity = sp_cap;
    initialized = false;
    rec_host.clear(); spec_host.clear();
    return reset_state(err);
  }

  int sync_host_state(int64_t it_first, int64_t it_last, std::string& err) override {
    return drain(it_first, it_last, err);
  }
};

}  // namespace ffsgpu
