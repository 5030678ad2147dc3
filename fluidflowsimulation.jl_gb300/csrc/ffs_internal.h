// Internal definitions shared by the CUDA passes and the C-ABI host runtime.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/ffs.h"
#include "ffs_fft.cuh"

namespace ffsgpu {

// Field codes produced by the spectral prologue of the inverse z pass.
enum FieldCode : int {
  F_UX = 0, F_UY, F_UZ,          // velocity
  F_WX, F_WY, F_WZ,              // vorticity  i k x u
  F_SXX, F_SXY, F_SXZ, F_SYY, F_SYZ,   // strain sym(i k (x) u), traceless, 5 comps
  F_RHO,                         // density perturbation
  // dynamic Smagorinsky: the test-filtered velocity G u and strain G S (fourierspacep1!,
  // models.jl:99-103), G = exp(-D^2 k^2 / 24) with the test filter width D
  F_GUX, F_GUY, F_GUZ,
  F_GSXX, F_GSXY, F_GSXZ, F_GSYY, F_GSYZ,
  F_GWX, F_GWY, F_GWZ,           // and with the dynamic P tensor the filtered vorticity G w
  F_GRX, F_GRY, F_GRZ            // the fourth field's gradient i k rho (its LES diffusion)
};

// Forward-field roles consumed by the forward z pass.
enum FwdRole : int { R_NX = 0, R_NY, R_NZ, R_KE, R_TXX, R_TXY, R_TXZ, R_TYY, R_TYZ, R_FX, R_FY, R_FZ };

// Spectrum fields of write_spec (spec.jl:1-171), in record order. The velocity-only
// fields always come first; LES, hyperviscosity and density add theirs.
enum SpecField : int {
  SF_U_H = 0, SF_U_V, SF_VIS_H, SF_VIS_V, SF_NL_H, SF_NL_V, SF_PRESS_H, SF_PRESS_V, SF_BASE_COUNT
};
constexpr int SPEC_MAX_FIELDS = 32;

// Stats partial-sum quantities (per CTA of the forward z pass).
enum StatQ : int {
  Q_U1 = 0, Q_U2, Q_U3, Q_U12, Q_U22, Q_U32, Q_EH, Q_EV, Q_NLH, Q_NLV, Q_PH, Q_PV,
  Q_D1DY, Q_D1DX, Q_D2DY, Q_D2DX, Q_LESH, Q_LESV, Q_HVH, Q_HVV,
  Q_RHO, Q_RHO2, Q_DR1, Q_DR2, Q_DR3, Q_BF, Q_HP, Q_VP,
  Q_IL0,  // 9 integral-length plane sums: [component][plane x,y,z]
  // the same sums weighted by the squared Gaussian filter (Stats_fil.txt); Q_FDR1 keeps
  // only the last retained kx of each line, as the reference's filtered dx_squared_mean
  Q_FU12 = Q_IL0 + 9, Q_FU22, Q_FU32, Q_FEH, Q_FEV, Q_FNLH, Q_FNLV, Q_FLESH, Q_FLESV, Q_FHVH, Q_FHVV,
  Q_FRHO2, Q_FDR1, Q_FDR2, Q_FDR3, Q_FBF,
  Q_RHV, Q_FRHV,   // density hyperviscous sum (rhohdiss) and its filtered twin
  Q_RPR, Q_FRPR,   // density LES transfer (rhopr: proj(i k . flux, rho)) and its filtered twin
  Q_COUNT
};
constexpr int QPAD = 64;
constexpr int FFS_PF_MAXSH = 520;   // 2D shells of the kz = 0 plane forcing: min(nx/2+1, ny/2) <= 513

// Device-resident scalar state (one per simulation).
struct DevState {
  long long iteration;     // reference s.iteration
  double time;             // reference s.time
  double dt, dt2, dt3;     // integrator dt history (dt = current)
  long long ts_iter;       // integrator's own call counter
  double At, Bt, Ct;       // AB3 scalars of the current step
  int stage;               // 1, 2, 3: integrator stage of the current step
  int hist_parity;         // which history slot holds fm1
  double slot_u;           // the reference's reductionh[1] (single Julia thread)
  double slot_rho;         // density reduction[1]
  unsigned long long umax_bits;    // running max |u_i| of this step (atomicMax on double bits)
  unsigned long long rhomax_bits;  // running max |rho|
  double force_coef;       // isotropic band forcing: eps / (2 E_f)
  double Ef;
  double pf_hp, pf_vp;     // kz = 0 plane forcing: horizontal and vertical power of the last call
  double nl_h, nl_v, press_h, press_v;  // last non-linear / pressure stats
  double nl_hf, nl_vf, press_hf, press_vf;  // their filtered twins (Stats_fil.txt)
  double dyn_dtm1;         // piomelliSmagorinsky: dt of its previous coefficient (dtm1)
  double dyn_dtpm1;        // piomelliSandP: dt of its previous cp (dtpm1)
  long long nrec;          // stats records written
  long long nspec;         // spectrum records written
  unsigned int err;        // bit 0: non-finite value in the update
  int pad0;
  // per-step update scalars in both precisions, written by the scalar kernel:
  // At, Bt, Ct, fix_fm2 factor -(dt3+dt2)/dt2, forcing increment dt*eps/(2 E_f)
  double coef_d[5];
  float coef_f[6];
  int skip_table;          // 1: the ETD table of the previous step still holds (fixed dt, stage 3)
  int pad1;
};
enum CoefIdx : int { CO_A = 0, CO_B, CO_C, CO_FIX2, CO_FDT };
template <typename T> __device__ __forceinline__ T step_coef(const DevState* S, int i);
template <> __device__ __forceinline__ float step_coef<float>(const DevState* S, int i) { return S->coef_f[i]; }
template <> __device__ __forceinline__ double step_coef<double>(const DevState* S, int i) { return S->coef_d[i]; }

template <typename T> struct Inst {
  // grid
  int nx, ny, nz, nxh;
  int Mx, KXP;             // retained kx count, padded row length
  int NYR, ypos;           // retained ky count, count of retained ky >= 0
  int NZR, zpos;
  int uniformL;            // lx == ly == lz: ETD coefficients tabulated by i^2+j^2+l^2
  double lx, ly, lz;
  double inv_n;            // 1 / (nx ny nz)
  FftPlan px, py, pz;
  const cplx<T>* twx;
  const cplx<T>* twy;
  const cplx<T>* twz;
  const cplx<T>* twx_r;     // register-pass twiddles of the fused x pass, [m][i] = (c, c, s, s) of tw[i m]
  int x_pf_dist;            // fused x pass: CTAs resident at once (the CTA that many ahead
                            // gets its input prefetched into L2); 0: no prefetch
  // resident spectral state, compact [comp][kz'][ky'][KXP]
  cplx<T>* uh;             // 3 velocity comps (+ rho)
  cplx<T>* hist;           // [2][ncomp][...]
  long long cstride;       // elements per compact component = NZR*NYR*KXP
  FastDiv fd_kxp, fd_nyr;  // index decomposition of the compact layout
  int ncomp;               // 3 or 4
  // work arrays
  cplx<T>* wz;             // [slot][nz][NYR][KXP]
  cplx<T>* wy;             // [slot][nz][ny][KXP]
  long long wzs, wys;      // slot strides
  double* phys;            // FP64 physical staging [field][nz][ny][nx]
  double* obuf;            // output capture (set only for the capture step's x pass)
  // scalar state and outputs
  DevState* st;
  double* partials;        // [stats CTAs][QPAD]
  cplx<T>* sbuf;           // scratch: N(3), ke, i k.tau(3), i k.flux (compact layout)
  double* records;         // stats records [cap][ncols]
  int rec_cap, ncols;
  double* spec;            // spectrum records [cap][4][nbin]
  int spec_cap, nbinH, nbinV;
  int nspecf;              // spectrum fields per record (each binned into H and V)
  double maxdkh, dkz;
  // ETD coefficient tables [q][4] (E, A, B, C), velocity then density
  T* etab;
  T* etab_rho;
  int qmax;
  // physics
  double nu, cfl, dt0;
  int ab3, adaptive, ref_slot;   // ab3: an explicit integrator (AB3 or Euler)
  int euler;               // Euller: u += dt rhs, dt as set_dt! gives it
  int hv, hv_m;
  double hv_nu;
  int hv_kind;             // 0 nuh k^2M, 1 the spectral barrier (hv_initk, hv_endk)
  double hv_initk, hv_endk;
  int rho_les;             // LES of the fourth field: 0 none, 1 eddy diffusion, 2 vorticity diffusion
  double rho_les_c;        //   c Delta^2 / 2 of the vorticity term
  int rho_hv, rho_hv_m;    // density hyperviscosity: 0 none, 1 rho_hv_nu k^2M, 2 the spectral barrier
  double rho_hv_nu, rho_hv_initk, rho_hv_endk;
  int les;
  double les_alpha;        // c^2 Delta^2
  int les_model;           // FFS_LES_* (Smagorinsky, Vreman, production, Silvis, stable non-linear)
  double les_c, les_d2;    // the model's constant c and Delta^2
  double les_cp;           // Silvis P constant
  double les_cb;           // SandP: cb (0: no P term)
  int dyn;                 // dynamic Smagorinsky (FFS_LES_DYNAMIC or FFS_LES_PIOMELLI)
  int piom;                //   piomelliSmagorinsky: extrapolated coefficient in Sa
  double* dyn_cm1;         //   its coefficient of the previous step [z][y][x]
  int dynp;                //   dynamic P tensor: 1 dynamicSandP, 2 piomelliSandP (cp: dyn_c's second plane)
  double* dyn_cpm1;        //   piomelliSandP's cp of the previous step
  double dyn_d2h;          //   test filter width^2
  double les_cmin;         //   smallest coefficient kept (cmin)
  int sfil;                // filtered stats and spectra (specFil)
  double fil_d2;           //   filter width^2 (SPEC_FIL_D2)
  const double* dyn_c;     //   averaged coefficient in physical space [z][y][x]
  int density, gdir;      // density: a fourth field (density, or with scalar the passive scalar)
  int scalar;              // the fourth field is a passive scalar: no buoyancy, no CFL cap, own stats
  double alpha, dgrad, gval;
  int forcing;
  double f_eps, f_kf;
  // kz = 0 plane forcing (FFS_PF_*): per-shell state and tables, plane-mode lists, force
  int pforce, pf_nsh;
  double pf_maxdk, pf_kf, pf_tf, pf_alpha, pf_cfl;
  double* pf_d;            // [9][nsh]: R, Em, factor, avgK, Zf, Qf power spectrum, N, Nm1, Ef;
                           // then aForcing's [4][NYR * KXP]: R, Em, factor, Zf per plane mode
  const int* pf_start;     // [nsh + 1]: retained kz = 0 modes of each spectrum shell (CSR)
  const int* pf_modes;     //   their plane index jc * KXP + ix
  const int* pf_nmode;     // [NYR * KXP]: forcing shell of each plane mode (-1: not forced;
                           // aForcing: 0 for the forced modes)
  cplx<T>* pf_force;       // [2][NYR * KXP] force on the kz = 0 plane, then [2][10] (0, 0, kz) modes
  int dt_stat, dt_spec;
  // the same constants in the arithmetic type (no per-element conversions)
  T Lx_t, Ly_t, Lz_t, iLx_t, iLy_t, iLz_t;
  T inv_n_t, nu_t, hvnu_t, alpha_t, gval_t, dgrad_t, kf2_t;
  T inv_n2_t;              // 1/(2N): the step's forward z scale (the x pass leaves out its unpack 1/2)
  // field lists for the passes
  int wz_derived;          // FP64: the y pass forms w_z = i (kx Uy - ky Ux) from the z-transformed
                           // u (no kz in it), so the z pass skips one transform
  int nin;                 // inverse fields
  int in_code[12];
  int nout;                // forward fields (incl. kinetic-energy field)
  int out_role[12];
  int out_slot[12];
};

}  // namespace ffsgpu
