// The GPU passes of one pseudo-spectral step (templated on the arithmetic type T).
//
// Step = inverse z (spectral prologue) -> inverse y -> fused x pass (c2r, physical
// products, r2c) -> forward y -> scalar kernel (dt, integrator coefficients, forcing)
// -> forward z + update (projection, integrator, forcing, stats) -> finalize.
//
// Memory layout in HBM (complex T, kx fastest, kx padded to KXP):
//   uh   [comp][kz'][ky'][kx]     retained (dealiased) modes only
//   wz   [slot][z][ky'][kx]       after the z pass (inverse) / before it (forward)
//   wy   [slot][z][y][kx]         after the y pass (inverse) / before it (forward)
// Physical space exists only in shared memory inside the x pass.
#pragma once
#include <type_traits>
#include "ffs_ddmath.cuh"
#include "ffs_internal.h"

namespace ffsgpu {

// CTAs of at most 512 threads (<= 128 registers per thread); tiles shrink for large n.
#define FFS_MAXT 512

constexpr int LYZ_IO = 4;  // (y,z) lines per CTA in the transform-only x kernels

struct FieldList {
  int n;
  int code[28];   // FieldCode (inverse z) or role (forward passes): at most 15 + 11 filtered
  int slot[28];   // work-array slot
};

// Block coordinates of one unit of work: the launch's own (single simulation) or an
// entry of a batch work table (many simulations in one launch).
struct Blk {
  int x, y, z, nx;   // block index, and the number of blocks along x for grid-stride loops
  __device__ static Blk here() { return Blk{(int)blockIdx.x, (int)blockIdx.y, (int)blockIdx.z, (int)gridDim.x}; }
};

// ------------------------------------------------------------------ index helpers
template <typename T> __device__ __forceinline__ int ycomp(const Inst<T>& I, int y) {
  if (y < I.ypos) return y;
  int neg = I.NYR - I.ypos;
  if (y >= I.ny - neg) return y - (I.ny - I.NYR);
  return -1;
}
template <typename T> __device__ __forceinline__ int zcomp(const Inst<T>& I, int z) {
  if (z < I.zpos) return z;
  int neg = I.NZR - I.zpos;
  if (z >= I.nz - neg) return z - (I.nz - I.NZR);
  return -1;
}
// signed integer wavenumber index of compact y / z index
template <typename T> __device__ __forceinline__ int ysig(const Inst<T>& I, int jc) {
  int y = jc < I.ypos ? jc : I.ny - I.NYR + jc;
  return y < I.ny / 2 ? y : y - I.ny;
}
template <typename T> __device__ __forceinline__ int zsig(const Inst<T>& I, int kc) {
  int z = kc < I.zpos ? kc : I.nz - I.NZR + kc;
  return z < I.nz / 2 ? z : z - I.nz;
}

// asynchronous global -> shared copy of one complex element (8 or 16 bytes)
template <typename T> __device__ __forceinline__ void cp_async_elem(cplx<T>* dst, const cplx<T>* src) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(dst);
  if (sizeof(cplx<T>) == 16)
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(src) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// Bulk prefetch of [p, p + bytes) from global memory into L2 (no registers, no shared
// memory; p 16-byte aligned, bytes a multiple of 16).
__device__ __forceinline__ void prefetch_l2(const void* p, unsigned bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;\n" ::"l"(p), "r"(bytes) : "memory");
}

// wavenumber i / L: FP64 divides exactly like the reference (KX[i] = i/LX); FP32
// multiplies by the reciprocal.
template <typename T> __device__ __forceinline__ T kval(int i, T L, T iL) {
  return sizeof(T) == 8 ? T(i) / L : T(i) * iL;
}

// compact index g -> (ix, jc, kc)
template <typename T> __device__ __forceinline__ void decomp(const Inst<T>& I, unsigned g, int& ix, int& jc, int& kc) {
  const unsigned r = fdiv(g, I.fd_kxp);
  ix = (int)(g - r * I.fd_kxp.d);
  const unsigned q = fdiv(r, I.fd_nyr);
  jc = (int)(r - q * I.fd_nyr.d);
  kc = (int)q;
}

__device__ __forceinline__ void atomic_max_pos(unsigned long long* a, double v) {
  // non-negative doubles order like their bit patterns
  atomicMax(a, (unsigned long long)__double_as_longlong(v));
}

template <typename T> __device__ __forceinline__ double proj(cplx<T> a, cplx<T> b) {
  return (double)a.x * (double)b.x + (double)a.y * (double)b.y;
}

// ====================================================================================
// Inverse z pass with the spectral prologue (fourierspacep1!, models.jl:63-119):
//   velocity, vorticity i k x u, strain sym(i k (x) u), density, each to its own slot.
// grid (nfields, KXP/TX, NYR); block TX * tpl_z
// ====================================================================================
template <typename T, int TX, int N = 0>
__device__ __forceinline__ void b_inv_z(const Inst<T>& I, const FieldList& F, const Blk bk) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cplx<T>* s0 = reinterpret_cast<cplx<T>*>(smem_raw);
  cplx<T>* s1 = s0 + srows(I.nz) * TX;   // used by plans of three or more passes
  const int fi = bk.x, kx0 = bk.y * TX, jc = bk.z;
  const int code = F.code[fi];
  const long long cs = I.cstride;
  const int rowstride = I.NYR * I.KXP;
  const cplx<T>* uh = I.uh + (long long)jc * I.KXP + kx0;
  const T kyv = kval(ysig(I, jc), I.Ly_t, I.iLy_t);
  const T Lx = I.Lx_t, iLx = I.iLx_t, Lz = I.Lz_t, iLz = I.iLz_t;
  // The field's prologue is one of three forms, fixed per CTA (so each form gets its own
  // FFT with a branch-free loader): a copy of a component, a curl component
  // i (k_b u_c - k_c u_b), or a strain component (i/2)(k_a u_b + k_b u_a); the dynamic
  // model adds the copy and the strain times the test filter G (families 3 and 4).
  int fam, ca = 0, cb = 0;
  switch (code) {
    case F_GUX: case F_GUY: case F_GUZ: fam = 3; ca = code - F_GUX; break;
    case F_GSXX: fam = 4; ca = 0; cb = 0; break;
    case F_GSXY: fam = 4; ca = 0; cb = 1; break;
    case F_GSXZ: fam = 4; ca = 0; cb = 2; break;
    case F_GSYY: fam = 4; ca = 1; cb = 1; break;
    case F_GSYZ: fam = 4; ca = 1; cb = 2; break;
    case F_GRX: case F_GRY: case F_GRZ: fam = 6; ca = code - F_GRX; break;
    case F_GWX: fam = 5; ca = 1; cb = 2; break;
    case F_GWY: fam = 5; ca = 2; cb = 0; break;
    case F_GWZ: fam = 5; ca = 0; cb = 1; break;
    case F_UX: fam = 0; ca = 0; break;
    case F_UY: fam = 0; ca = 1; break;
    case F_UZ: fam = 0; ca = 2; break;
    case F_RHO: fam = 0; ca = 3; break;
    case F_WX: fam = 1; ca = 1; cb = 2; break;
    case F_WY: fam = 1; ca = 2; cb = 0; break;
    case F_WZ: fam = 1; ca = 0; cb = 1; break;
    case F_SXX: fam = 2; ca = 0; cb = 0; break;
    case F_SXY: fam = 2; ca = 0; cb = 1; break;
    case F_SXZ: fam = 2; ca = 0; cb = 2; break;
    case F_SYY: fam = 2; ca = 1; cb = 1; break;
    default: fam = 2; ca = 1; cb = 2; break;   // F_SYZ
  }
  const long long oa = ca * cs, ob = cb * cs;
  // wavenumber of axis d at (kx0 + l, jc, kc)
  auto kax = [&](int d, int l, int kc) -> T {
    return d == 0 ? kval(kx0 + l, Lx, iLx) : (d == 1 ? kyv : kval(zsig(I, kc), Lz, iLz));
  };
  cplx<T>* out = I.wz + (long long)F.slot[fi] * I.wzs + (long long)jc * I.KXP + kx0;
  auto st = [&](int l, int z, cplx<T> v) { out[(long long)z * rowstride + l] = v; };
  if (fam == 0) {
    auto ld = [&](int l, int z) -> cplx<T> {
      const int kc = zcomp(I, z);
      if (kc < 0 || kx0 + l >= I.Mx) return mk(T(0), T(0));
      return uh[oa + (long long)kc * rowstride + l];
    };
    fft_lines_n<+1, TX, T, N>(I.pz, s0, s1, TX, I.twz, ld, st);
  } else if (fam == 1) {
    auto ld = [&](int l, int z) -> cplx<T> {   // i (k_b u_c - k_c u_b), (b, c) = (ca, cb)
      const int kc = zcomp(I, z);
      if (kc < 0 || kx0 + l >= I.Mx) return mk(T(0), T(0));
      const long long o = (long long)kc * rowstride + l;
      const cplx<T> ub = uh[oa + o], uc = uh[ob + o];
      const T kb = kax(ca, l, kc), kc_ = kax(cb, l, kc);
      return mk(-(kb * uc.y - kc_ * ub.y), kb * uc.x - kc_ * ub.x);
    };
    fft_lines_n<+1, TX, T, N>(I.pz, s0, s1, TX, I.twz, ld, st);
  } else if (fam == 6) {
    auto ld = [&](int l, int z) -> cplx<T> {   // i k_a rho (fourierspacep1!, models.jl:110-112)
      const int kc = zcomp(I, z);
      if (kc < 0 || kx0 + l >= I.Mx) return mk(T(0), T(0));
      const cplx<T> r = uh[3 * cs + (long long)kc * rowstride + l];
      const T ka = kax(ca, l, kc);
      return mk(-ka * r.y, ka * r.x);
    };
    fft_lines_n<+1, TX, T, N>(I.pz, s0, s1, TX, I.twz, ld, st);
  } else if (fam == 2) {
    auto ld = [&](int l, int z) -> cplx<T> {   // (i/2)(k_a u_b + k_b u_a), (a, b) = (ca, cb)
      const int kc = zcomp(I, z);
      if (kc < 0 || kx0 + l >= I.Mx) return mk(T(0), T(0));
      const long long o = (long long)kc * rowstride + l;
      const cplx<T> ua = uh[oa + o], ub = uh[ob + o];
      const T ka = kax(ca, l, kc), kb = kax(cb, l, kc);
      const cplx<T> q = mk(ka * ub.x + kb * ua.x, ka * ub.y + kb * ua.y);
      return mk(-T(0.5) * q.y, T(0.5) * q.x);
    };
    fft_lines_n<+1, TX, T, N>(I.pz, s0, s1, TX, I.twz, ld, st);
  } else {
    // Gaussfilter (utils.jl:220-225): exp(-D^2 k.k / 24), k.k = kx kx + (ky ky + kz kz)
    const T aux = T(-I.dyn_d2h / 24.0);
    auto gk = [&](int l, int kc) -> T {
      const T kx = kax(0, l, kc), kz = kax(2, l, kc);
      return exp(aux * (kx * kx + (kyv * kyv + kz * kz)));
    };
    if (fam == 3) {
      auto ld = [&](int l, int z) -> cplx<T> {
        const int kc = zcomp(I, z);
        if (kc < 0 || kx0 + l >= I.Mx) return mk(T(0), T(0));
        return scl(uh[oa + (long long)kc * rowstride + l], gk(l, kc));
      };
      fft_lines_n<+1, TX, T, N>(I.pz, s0, s1, TX, I.twz, ld, st);
    } else if (fam == 5) {
      auto ld = [&](int l, int z) -> cplx<T> {   // G i (k_b u_c - k_c u_b)
        const int kc = zcomp(I, z);
        if (kc < 0 || kx0 + l >= I.Mx) return mk(T(0), T(0));
        const long long o = (long long)kc * rowstride + l;
        const cplx<T> ub = uh[oa + o], uc = uh[ob + o];
        const T kb = kax(ca, l, kc), kc_ = kax(cb, l, kc);
        const T g = gk(l, kc);
        return mk(g * (-(kb * uc.y - kc_ * ub.y)), g * (kb * uc.x - kc_ * ub.x));
      };
      fft_lines_n<+1, TX, T, N>(I.pz, s0, s1, TX, I.twz, ld, st);
    } else {
      auto ld = [&](int l, int z) -> cplx<T> {   // G (i/2)(k_a u_b + k_b u_a)
        const int kc = zcomp(I, z);
        if (kc < 0 || kx0 + l >= I.Mx) return mk(T(0), T(0));
        const long long o = (long long)kc * rowstride + l;
        const cplx<T> ua = uh[oa + o], ub = uh[ob + o];
        const T ka = kax(ca, l, kc), kb = kax(cb, l, kc);
        const cplx<T> q = mk(ka * ub.x + kb * ua.x, ka * ub.y + kb * ua.y);
        const T g = gk(l, kc);
        return mk(g * (-T(0.5) * q.y), g * (T(0.5) * q.x));
      };
      fft_lines_n<+1, TX, T, N>(I.pz, s0, s1, TX, I.twz, ld, st);
    }
  }
}
// with a compile-time plan the CTA has exactly TX * ct_tpl threads; the register cap
// lets 9 CTAs share an SM
template <typename T, int TX, int N = 0>
__global__ void __launch_bounds__(N > 0 ? TX * ct_tpl<(N > 0 ? N : 128)>() : FFS_MAXT, N > 0 ? 9 : 1)
k_inv_z(Inst<T> I, FieldList F) {
  b_inv_z<T, TX, N>(I, F, Blk::here());
}

// ====================================================================================
// Inverse y pass: grid (nfields, KXP/TX, nz); block TX * tpl_y
// ====================================================================================
template <typename T, int TX, int N = 0>
__device__ __forceinline__ void b_inv_y(const Inst<T>& I, const FieldList& F, const Blk bk) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cplx<T>* s0 = reinterpret_cast<cplx<T>*>(smem_raw);
  cplx<T>* s1 = s0 + srows(I.ny) * TX;
  const int fi = bk.x, kx0 = bk.y * TX, z = bk.z;
  const cplx<T>* in = I.wz + (long long)F.slot[fi] * I.wzs + (long long)z * I.NYR * I.KXP + kx0;
  cplx<T>* out = I.wy + (long long)F.slot[fi] * I.wys + (long long)z * I.ny * I.KXP + kx0;
  auto st = [&](int l, int y, cplx<T> v) { out[(long long)y * I.KXP + l] = v; };
  if constexpr (sizeof(T) == 8) {
    const int code = F.code[fi];
    if (I.wz_derived && (code == F_WZ || code == F_SXX || code == F_SXY || code == F_SYY)) {
      // w_z = i (kx u_y - ky u_x) and the strain components xx, xy, yy have no kz: formed
      // here from the z-transformed u_x, u_y (slots 0 and 1), with the spectral prologue's
      // expressions. The wavenumbers come from a table after the FFT buffers (no FP64
      // conversions per element).
      T* ktab = reinterpret_cast<T*>(s0 + (size_t)srows(I.ny) * TX * (I.py.np >= 3 ? 2 : 1));   // [TX] kx, [NYR] ky
      for (int t = threadIdx.x; t < TX + I.NYR; t += blockDim.x)
        ktab[t] = t < TX ? kval(kx0 + t, I.Lx_t, I.iLx_t) : kval(ysig(I, t - TX), I.Ly_t, I.iLy_t);
      __syncthreads();
      const long long o = (long long)z * I.NYR * I.KXP + kx0;
      const cplx<T>* ux = I.wz + o;
      const cplx<T>* uy = I.wz + I.wzs + o;
      auto ldw = [&](int l, int y) -> cplx<T> {
        const int jc = ycomp(I, y);
        if (jc < 0) return mk(T(0), T(0));
        const cplx<T> a = ux[(long long)jc * I.KXP + l], b = uy[(long long)jc * I.KXP + l];
        const T kx = ktab[l], ky = ktab[TX + jc];
        if (code == F_WZ) return mk(-(kx * b.y - ky * a.y), kx * b.x - ky * a.x);
        // (i/2)(k_a u_b + k_b u_a) with (a, b) = (x, x), (x, y), (y, y)
        const T k1 = code == F_SYY ? ky : kx, k2 = code == F_SXX ? kx : ky;
        const cplx<T> v1 = code == F_SXX ? a : b, v2 = code == F_SYY ? b : a;
        const cplx<T> q = mk(k1 * v1.x + k2 * v2.x, k1 * v1.y + k2 * v2.y);
        return mk(-T(0.5) * q.y, T(0.5) * q.x);
      };
      fft_lines_n<+1, TX, T, N>(I.py, s0, s1, TX, I.twy, ldw, st);
      return;
    }
  }
  auto ld = [&](int l, int y) -> cplx<T> {
    const int jc = ycomp(I, y);
    if (jc < 0) return mk(T(0), T(0));
    return in[(long long)jc * I.KXP + l];
  };
  fft_lines_n<+1, TX, T, N>(I.py, s0, s1, TX, I.twy, ld, st);
}
template <typename T, int TX, int N = 0>
__global__ void __launch_bounds__(FFS_MAXT) k_inv_y(Inst<T> I, FieldList F) {
  b_inv_y<T, TX, N>(I, F, Blk::here());
}

// ====================================================================================
// Forward y pass (keeps retained ky only): grid (nfields, KXP/TX, nz)
// The kinetic-energy field is transformed only at stats/spectrum iterations.
// ====================================================================================
template <typename T, int TX, int N = 0>
__device__ __forceinline__ void b_fwd_y(const Inst<T>& I, const FieldList& F, const Blk bk) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cplx<T>* s0 = reinterpret_cast<cplx<T>*>(smem_raw);
  cplx<T>* s1 = s0 + srows(I.ny) * TX;
  const int fi = bk.x, kx0 = bk.y * TX, z = bk.z;
  if (F.code[fi] == R_KE) {
    const long long it = I.st->iteration;
    if ((it % I.dt_stat) != 0 && (it % I.dt_spec) != 0) return;
  }
  const cplx<T>* in = I.wy + (long long)F.slot[fi] * I.wys + (long long)z * I.ny * I.KXP + kx0;
  cplx<T>* out = I.wz + (long long)F.slot[fi] * I.wzs + (long long)z * I.NYR * I.KXP + kx0;
  auto ld = [&](int l, int y) -> cplx<T> { return in[(long long)y * I.KXP + l]; };
  auto st = [&](int l, int y, cplx<T> v) {
    const int jc = ycomp(I, y);
    if (jc >= 0) out[(long long)jc * I.KXP + l] = v;
  };
  fft_lines_n<-1, TX, T, N>(I.py, s0, s1, TX, I.twy, ld, st);
}
template <typename T, int TX, int N = 0>
__global__ void __launch_bounds__(FFS_MAXT) k_fwd_y(Inst<T> I, FieldList F) {
  b_fwd_y<T, TX, N>(I, F, Blk::here());
}

// ====================================================================================
// Fused x pass (realspace! + realspacecalculation! + calc_les! + find_max, models.jl
// 121-214 / 228-280, les_real_calc.jl:13-139, utils.jl:247-258):
//   stage half spectra -> c2r (two real fields per complex line) -> physical products
//   -> r2c (two real fields per complex line) -> Hermitian unpack -> store kx < KXP.
// grid (ny*nz/LYZ); block >= LYZ*PIN*tpl_x
// Real fields in:  u(3) w(3) [S(5) if LES] [rho if DEN] [grad rho(3) if DEN == 2]
// Real fields out: N(3) ke [tau(5) if LES] [flux(3) if DEN]
// DEN: 0 no fourth field, 1 density / scalar, 2 with its LES diffusion (needs LES)
// ====================================================================================
// Running max of |x| (find_max, utils.jl:247-258). FP64: on the bit patterns, which order
// non-negative doubles like their values, so the integer pipe does the work and the FP64
// pipe (the bound of the FP64 passes) does none; FP32: fmaxf.
template <typename T> struct AbsMax;
template <> struct AbsMax<float> {
  float v = 0.f;
  __device__ __forceinline__ void add(float x) { v = fmaxf(v, fabsf(x)); }
  __device__ __forceinline__ float get() const { return v; }
};
template <> struct AbsMax<double> {
  unsigned long long b = 0ull;
  __device__ __forceinline__ void add(double x) {
    const unsigned long long a = (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffull;
    b = a > b ? a : b;
  }
  __device__ __forceinline__ double get() const { return __longlong_as_double((long long)b); }
};

// Block-wide max of |u_i| (and |rho|) in T, then one atomicMax per CTA on the state.
// red: shared scratch of at least 32 T per quantity.
template <typename T, bool DEN>
__device__ __forceinline__ void block_max_to_state(const Inst<T>& I, T umax, T rmax, T* red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    umax = fmax(umax, __shfl_xor_sync(0xffffffffu, umax, o));
    if (DEN) rmax = fmax(rmax, __shfl_xor_sync(0xffffffffu, rmax, o));
  }
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = (blockDim.x + 31) >> 5;
  if (lane == 0) { red[w] = umax; if (DEN) red[32 + w] = rmax; }
  __syncthreads();
  if (threadIdx.x == 0) {
    T m = T(0), r = T(0);
    for (int i = 0; i < nw; ++i) { m = fmax(m, red[i]); if (DEN) r = fmax(r, red[32 + i]); }
    atomic_max_pos(&I.st->umax_bits, (double)m);
    if (DEN) atomic_max_pos(&I.st->rhomax_bits, (double)r);
  }
}

// tau of the pointwise LES models other than plain Smagorinsky (calc_les!,
// les_real_calc.jl:13-139), from the strain S (traceless: xx, xy, xz, yy, yz) and the
// vorticity w at one point. Om = AntiSymTen(w/2) is the rotation tensor (FluidTensors'
// AntiSymTen(v) is taken as the cross-product matrix of v); Lie(A, B) = A B - B A.
//   Vreman (VremanLESModel.jl): a = S - Om = grad u^T, beta = D^2 a^T a,
//     nu_t = c sqrt(max(B_beta, 0) / a:a), tau = 2 nu_t S
//   production viscosity (ProductionViscosityLESModel.jl): nu_t = max(0, c D^2 (Om^2:S - S^2:S) / (2 S:S))
//   Silvis (silvismodel.jl): f = |S w| / (|S| |w|), nu_t = c^2 D^2 f^3 |S| / 2, nu_p = cp D^2 f^4 / 4,
//     tau = 2 nu_t S + nu_p Lie(S, Om)
//   stable non-linear (stablenonlinearmodel.jl): T = traceless(Om^2 + Lie(S, Om) - S^2),
//     m = -min(0, c D^2 (Om^2:S - S^2:S) / (2 S:S)), tau = c D^2 T + 2 m S
//   SandP (les_real_calc.jl:104-111): tau += cb D^2 Lie(S, Om)
template <typename T>
__device__ __forceinline__ void les_model_tau(const Inst<T>& I, T xx, T xy, T xz, T yy, T yz, T wx, T wy, T wz,
                                              T* o, T& nut_out) {
  const T zz = -xx - yy;
  const T S[3][3] = {{xx, xy, xz}, {xy, yy, yz}, {xz, yz, zz}};
  const T p = T(0.5) * wx, q = T(0.5) * wy, r = T(0.5) * wz;
  const T Om[3][3] = {{T(0), -r, q}, {r, T(0), -p}, {-q, p, T(0)}};
  const T c = T(I.les_c), d2 = T(I.les_d2);
  T t[3][3];
  T ss = T(0);
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) ss += S[i][j] * S[i][j];
  // Lie(S, Om) = S Om - Om S, Om^2, S^2
  T lie[3][3], om2[3][3], s2[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      T a = T(0), b = T(0), e = T(0), g = T(0);
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        a += S[i][k] * Om[k][j];
        b += Om[i][k] * S[k][j];
        e += Om[i][k] * Om[k][j];
        g += S[i][k] * S[k][j];
      }
      lie[i][j] = a - b;
      om2[i][j] = e;
      s2[i][j] = g;
    }
  T om2s = T(0), s2s = T(0);
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) { om2s += om2[i][j] * S[i][j]; s2s += s2[i][j] * S[i][j]; }
  const int m = I.les_model;
  if (m == FFS_LES_VREMAN) {
    T a[3][3], aa = T(0);
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) { a[i][j] = S[i][j] - Om[i][j]; aa += a[i][j] * a[i][j]; }
    T b[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        T v = T(0);
#pragma unroll
        for (int k = 0; k < 3; ++k) v += a[k][i] * a[k][j];
        b[i][j] = d2 * v;
      }
    T B = b[0][0] * (b[1][1] + b[2][2]) + b[1][1] * b[2][2] - (b[0][1] * b[0][1] + b[0][2] * b[0][2] + b[1][2] * b[1][2]);
    B = B < T(0) ? T(0) : B;
    const T nut = c * sqrt(B / aa);
    nut_out = nut;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) t[i][j] = T(2) * nut * S[i][j];
  } else if (m == FFS_LES_PRODUCTION) {
    const T qv = c * d2 * (om2s - s2s) / (T(2) * ss);
    const T nut = ss == T(0) ? T(0) : (qv > T(0) ? qv : T(0));
    nut_out = nut;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) t[i][j] = T(2) * nut * S[i][j];
  } else if (m == FFS_LES_SILVIS) {
    T sw[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) sw[i] = S[i][0] * wx + S[i][1] * wy + S[i][2] * wz;
    const T fv = sqrt(sw[0] * sw[0] + sw[1] * sw[1] + sw[2] * sw[2]) / (sqrt(ss) * sqrt(wx * wx + wy * wy + wz * wz));
    const T nut = c * c * d2 * fv * fv * fv * sqrt(ss) / T(2);
    const T nup = T(I.les_cp) * d2 * fv * fv * fv * fv / T(4);
    nut_out = nut;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) t[i][j] = T(2) * nut * S[i][j] + nup * lie[i][j];
  } else if (m == FFS_LES_STABLE_NL) {
    T tt[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) tt[i][j] = om2[i][j] + lie[i][j] - s2[i][j];
    const T tr = (tt[0][0] + tt[1][1] + tt[2][2]) / T(3);
    const T qv = c * d2 * (om2s - s2s) / (T(2) * ss);
    const T mnu = ss == T(0) ? T(0) : (qv < T(0) ? -qv : T(0));
    nut_out = ss == T(0) ? T(0) : (qv > T(0) ? qv : T(0));   // stable_nl_eddy_viscosity's nu
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) t[i][j] = c * d2 * (tt[i][j] - (i == j ? tr : T(0))) + T(2) * mnu * S[i][j];
  } else {   // Smagorinsky (with the SandP term below)
    const T nut = c * c * d2 * sqrt(ss);
    nut_out = nut;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) t[i][j] = T(2) * nut * S[i][j];
  }
  if (I.les_cb != 0.0) {
    const T beta = T(I.les_cb) * d2;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) t[i][j] += beta * lie[i][j];
  }
  o[0] = t[0][0]; o[1] = t[0][1]; o[2] = t[0][2]; o[3] = t[1][1]; o[4] = t[1][2];
}

template <bool LES, int DEN> struct XFields {
  static_assert(DEN != 2 || LES, "the fourth field's LES diffusion needs the LES model");
  static constexpr int nin = 6 + (LES ? 5 : 0) + (DEN ? 1 : 0) + (DEN == 2 ? 3 : 0);
  static constexpr int nout = 4 + (LES ? 5 : 0) + (DEN ? 3 : 0);
  static constexpr int PIN = (nin + 1) / 2;
  static constexpr int POUT = (nout + 1) / 2;
};

// DIAG (output iterations with output capture): also store the physical LES stress, the
// dynamic coefficients and the fourth field's LES flux to I.obuf (writeoutput,
// output.jl:22-42), as FP64 planes [field][z][y][x]: tau xx, xy, xz, yy, yz, then c
// (dynamic models), cp (dynamic P tensor), then the flux's 3 components (density LES)
template <typename T, bool LES, int DEN, int LYZ, int N = 0, bool DIAG = false>
__device__ __forceinline__ void b_x_pass(const Inst<T>& I, const Blk bk) {
  using XF = XFields<LES, DEN>;
  constexpr int PIN = XF::PIN, POUT = XF::POUT;
  constexpr int LIN = PIN * LYZ, LOUT = POUT * LYZ;
  constexpr int LSX = LIN + 1;   // odd line stride: conflict-free column reads in the unpack
  // with a compile-time plan the CTA has LIN * ct_tpl<N>() threads rounded up to whole warps
  constexpr int XNT = N > 0 ? ((LIN * ct_tpl<(N > 0 ? N : 128)>() + 31) / 32) * 32 : 0;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int n = I.nx, Mx = I.Mx;
  const int MXP = Mx | 1;
  // two buffers of [n][LSX] (the second at least as large as the staged half spectra,
  // which live in it: the first c2r pass reads them and writes the first buffer)
  cplx<T>* s0 = reinterpret_cast<cplx<T>*>(smem_raw);
  cplx<T>* s1 = s0 + (size_t)srows(n) * LSX;
  cplx<T>* stage = s1;                                                       // [nin][LYZ][MXP]
  __shared__ T red[64];

  const int g0 = bk.x * LYZ;
  const long long it = I.st->iteration;
  const bool want_ke = ((it % I.dt_stat) == 0) || ((it % I.dt_spec) == 0);

  // 1. stage the half spectra (coalesced along kx)
  {
    const int wv = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int row = wv; row < XF::nin * LYZ; row += nw) {   // row = f * LYZ + q
      const int q = row % LYZ, f = row / LYZ;
      const cplx<T>* src = I.wy + (long long)f * I.wys + (long long)(g0 + q) * I.KXP;
      cplx<T>* dst = stage + row * MXP;
      for (int kx = lane; kx < Mx; kx += 32) cp_async_elem(dst + kx, src + kx);
    }
    cp_async_wait_all();
  }
  __syncthreads();

  // 2. c2r: complex line l = p*LYZ + q carries fields (2p, 2p+1) of line q
  auto ldi = [&](int l, int j) -> cplx<T> {
    const int p = l / LYZ, q = l % LYZ;
    const bool cj = 2 * j > n;
    const int k = cj ? n - j : j;
    if (k >= Mx) return mk(T(0), T(0));
    const int fa = 2 * p, fb = 2 * p + 1;
    cplx<T> A = stage[(fa * LYZ + q) * MXP + k];
    cplx<T> B = fb < XF::nin ? stage[(fb * LYZ + q) * MXP + k] : mk(T(0), T(0));
    if (k == 0 || 2 * k == n) { A.y = T(0); B.y = T(0); }
    if (cj) { A.y = -A.y; B.y = -B.y; }
    return mk(A.x - B.y, A.y + B.x);
  };
  cplx<T>* ri = fft_result_buffer(I.px, s0, s1);   // physical values end up here
  auto sti = [&](int l, int j, cplx<T> v) { ri[sidx(j, l, LSX)] = v; };
  fft_lines_n<+1, LIN, T, N, decltype(ldi), decltype(sti), LSX, XNT>(I.px, s0, s1, LSX, I.twx, ldi, sti);

  // 3-5 twice, with and without the kinetic-energy field (output 3, needed only at stats
  // and spectrum iterations). Without it the other outputs pair up in order: output
  // index nk(t) of the t-th one; an odd one out of line q shares a complex line with
  // that of line q ^ 1 (LYZ >= 2), so no complex line carries a zero half.
  constexpr int NO = XF::nout, M_NK = NO - 1, P2 = M_NK / 2, ODD = M_NK % 2;
  constexpr int LOUT_NK = P2 * LYZ + (ODD ? (LYZ >= 2 ? LYZ / 2 : 1) : 0);
  static_assert(LOUT_NK <= LOUT && LOUT <= LIN, "output lines");
  auto nk = [](int t) { return t < 3 ? t : t + 1; };
  AbsMax<T> umaxt, rmaxt;
  const T les2 = T(2) * T(I.les_alpha);
  auto tail = [&](auto ke_c) {
  constexpr bool KE = decltype(ke_c)::value;
  // 3. physical space products: inputs from ri, outputs into s1
  for (int e = threadIdx.x; e < n * LYZ; e += blockDim.x) {
    const int q = e % LYZ, j = e / LYZ;
    const cplx<T>* row = ri + sidx(j, q, LSX);
    cplx<T>* orow = s1 + sidx(j, q, LSX);
    T f[2 * PIN];
#pragma unroll
    for (int p = 0; p < PIN; ++p) { cplx<T> v = row[p * LYZ]; f[2 * p] = v.x; f[2 * p + 1] = v.y; }
    const T ux = f[0], uy = f[1], uz = f[2], wx = f[3], wy = f[4], wz = f[5];
    T o[2 * POUT];
#pragma unroll
    for (int r = 0; r < 2 * POUT; ++r) o[r] = T(0);
    o[0] = uy * wz - uz * wy;             // (u x w), models.jl:260
    o[1] = uz * wx - ux * wz;
    o[2] = ux * wy - uy * wx;
    if (KE) o[3] = T(0.5) * (ux * ux + uy * uy + uz * uz);   // models.jl:224
    umaxt.add(ux); umaxt.add(uy); umaxt.add(uz);
    T nut = T(0);   // the model's eddy viscosity: the fourth field's eddy diffusivity
    if (LES) {
      const T xx = f[6], xy = f[7], xz = f[8], yy = f[9], yz = f[10];
      if (I.les_model == FFS_LES_SMAGORINSKY && I.les_cb == 0.0) {
        const T zz = -xx - yy;
        const T nrm = sqrt(xx * xx + yy * yy + zz * zz + T(2) * (xy * xy + xz * xz + yz * yz));
        const T two_nut = les2 * nrm;   // tau = 2 nu_t S, nu_t = c^2 D^2 |S|
        nut = T(0.5) * two_nut;         // exact: (2a) b = 2 (a b)
        o[4] = two_nut * xx; o[5] = two_nut * xy; o[6] = two_nut * xz; o[7] = two_nut * yy; o[8] = two_nut * yz;
      } else if (I.dyn) {
        // dynamic Smagorinsky (les_real_calc.jl:71-73): nu_t = max(cmin, min(0.4, c)) D^2 |S|,
        // c the averaged coefficient at this point (NaN kept, as Julia's min/max do)
        const T zz = -xx - yy;
        const T nrm = sqrt(xx * xx + yy * yy + zz * zz + T(2) * (xy * xy + xz * xz + yz * yz));
        const long long pi = (long long)(g0 + q) * n + j;
        T cc = T(I.dyn_c[pi]);
        if (!isnan(cc)) cc = fmax(T(I.les_cmin), fmin(T(0.4), cc));
        nut = cc * T(I.les_d2) * nrm;
        const T two_nut = T(2) * nut;
        o[4] = two_nut * xx; o[5] = two_nut * xy; o[6] = two_nut * xz; o[7] = two_nut * yy; o[8] = two_nut * yz;
        if (I.dynp || I.les_cb != 0.0) {
          // + max(-0.8, min(0.8, cp)) D^2 Lie(S, W) (les_real_calc.jl:104-106), or SandP's
          // cb D^2 Lie(S, W) (les_real_calc.jl:98-104)
          T b;
          if (I.dynp) {
            T cp = T(I.dyn_c[(long long)I.nx * I.ny * I.nz + pi]);
            if (!isnan(cp)) cp = fmax(T(-0.8), fmin(T(0.8), cp));
            b = cp * T(I.les_d2);
          } else {
            b = T(I.les_cb) * T(I.les_d2);
          }
          const T zz2 = -xx - yy;
          const T Sm[3][3] = {{xx, xy, xz}, {xy, yy, yz}, {xz, yz, zz2}};
          const T p_ = T(0.5) * wx, q_ = T(0.5) * wy, r_ = T(0.5) * wz;
          const T W[3][3] = {{T(0), -r_, q_}, {r_, T(0), -p_}, {-q_, p_, T(0)}};
          T lie[5];
          const int ii[5] = {0, 0, 0, 1, 1}, jj[5] = {0, 1, 2, 1, 2};
#pragma unroll
          for (int e2 = 0; e2 < 5; ++e2) {
            T a2 = T(0), b2 = T(0);
#pragma unroll
            for (int k = 0; k < 3; ++k) { a2 += Sm[ii[e2]][k] * W[k][jj[e2]]; b2 += W[ii[e2]][k] * Sm[k][jj[e2]]; }
            lie[e2] = a2 - b2;
          }
#pragma unroll
          for (int e2 = 0; e2 < 5; ++e2) o[4 + e2] += b * lie[e2];
        }
      } else {
        les_model_tau<T>(I, xx, xy, xz, yy, yz, wx, wy, wz, o + 4, nut);
      }
    }
    T lx = T(0), ly = T(0), lz = T(0);   // the fourth field's LES flux
    if (DEN) {
      constexpr int fr = LES ? 11 : 6, of = LES ? 9 : 4;
      const T rho = f[fr];
      rmaxt.add(rho);
      if (DEN == 2) {
        // calc_les! (les_real_calc.jl:116-134): nu_t grad rho (+ (c D^2 / 2) w x grad rho),
        // then realspacecalculation! adds it to -rho u (models.jl:265-268)
        constexpr int fg = fr + 1;
        const T gx = f[fg], gy = f[fg + 1], gz = f[fg + 2];
        lx = nut * gx; ly = nut * gy; lz = nut * gz;
        if (I.rho_les == 2) {
          const T cr = T(I.rho_les_c);
          lx += cr * (wy * gz - wz * gy); ly += cr * (wz * gx - wx * gz); lz += cr * (wx * gy - wy * gx);
        }
        o[of] = -rho * ux + lx; o[of + 1] = -rho * uy + ly; o[of + 2] = -rho * uz + lz;
      } else {
        o[of] = -rho * ux; o[of + 1] = -rho * uy; o[of + 2] = -rho * uz;   // models.jl:266
      }
    }
    if constexpr (DIAG && LES) {
      const long long npl = (long long)n * I.ny * I.nz, pi = (long long)(g0 + q) * n + j;
#pragma unroll
      for (int c = 0; c < 5; ++c) I.obuf[c * npl + pi] = (double)o[4 + c];
      int pl = 5;
      if (I.dyn) I.obuf[(pl++) * npl + pi] = I.dyn_c[pi];
      if (I.dynp) I.obuf[(pl++) * npl + pi] = I.dyn_c[npl + pi];
      if (DEN == 2 && !I.scalar) {
        I.obuf[pl * npl + pi] = (double)lx; I.obuf[(pl + 1) * npl + pi] = (double)ly;
        I.obuf[(pl + 2) * npl + pi] = (double)lz;
      }
    }
    if (KE) {
#pragma unroll
      for (int r = 0; r < POUT; ++r) orow[r * LYZ] = mk(o[2 * r], o[2 * r + 1]);
    } else {
#pragma unroll
      for (int r = 0; r < P2; ++r) orow[r * LYZ] = mk(o[nk(2 * r)], o[nk(2 * r + 1)]);
      if (ODD) {
        const T v = o[nk(M_NK - 1)];
        if (LYZ >= 2) reinterpret_cast<T*>(s1 + sidx(j, P2 * LYZ + q / 2, LSX))[q & 1] = v;
        else s1[sidx(j, P2 * LYZ, LSX)] = mk(v, T(0));
      }
    }
  }
  // block max -> one atomic per CTA (the max is exact in T; FP64 only for the atomic)
  if (I.adaptive) block_max_to_state<T, (DEN != 0)>(I, umaxt.get(), rmaxt.get(), red);
  __syncthreads();

  // 4. r2c of the output lines, result back into sx
  constexpr int LO = KE ? LOUT : LOUT_NK;
  cplx<T>* rf = fft_result_buffer(I.px, s0, s1);
  auto ldf = [&](int l, int j) -> cplx<T> { return s1[sidx(j, l, LSX)]; };
  auto stf = [&](int l, int j, cplx<T> v) { rf[sidx(j, l, LSX)] = v; };
  fft_lines_n<-1, LO, T, N, decltype(ldf), decltype(stf), LSX, XNT>(I.px, s0, s1, LSX, I.twx, ldf, stf);

  // 5. unpack A = (Z_k + conj Z_{n-k})/2, B = -i (Z_k - conj Z_{n-k})/2 and store
  const int KXP = I.KXP;
  {
    const int wv = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int l = wv; l < LO; l += nw) {
      // the outputs (oa, ob) and the (y,z) lines (qa, qb) of the two halves of line l;
      // with KE, line r * LYZ + q carries outputs (2r, 2r+1) of line q
      int oa, ob, qa, qb;
      if (KE) {
        oa = 2 * (l / LYZ); ob = oa + 1; qa = qb = l % LYZ;
      } else if (l < P2 * LYZ) {
        oa = nk(2 * (l / LYZ)); ob = nk(2 * (l / LYZ) + 1); qa = qb = l % LYZ;
      } else {
        const int t = l - P2 * LYZ;
        oa = ob = nk(M_NK - 1);
        qa = LYZ >= 2 ? 2 * t : 0;
        qb = LYZ >= 2 ? 2 * t + 1 : 0;
        if (LYZ < 2) ob = NO;   // (v, 0): no second half
      }
      const bool wa = oa < NO, wb = ob < NO;
      cplx<T>* da = I.wy + (long long)I.out_slot[wa ? oa : 0] * I.wys + (long long)(g0 + qa) * KXP;
      cplx<T>* db = I.wy + (long long)I.out_slot[wb ? ob : 0] * I.wys + (long long)(g0 + qb) * KXP;
      for (int k = lane; k < KXP; k += 32) {
        // 2A = Z_k + conj Z_{n-k}, 2B = -i (Z_k - conj Z_{n-k}): the factor 1/2 is in the
        // forward z pass's scale 1/(2N) (exact: a power of two through linear passes)
        cplx<T> A = mk(T(0), T(0)), B = mk(T(0), T(0));
        if (k < Mx) {
          const cplx<T> zk = rf[sidx(k, l, LSX)];
          const cplx<T> zm = rf[sidx(k == 0 ? 0 : n - k, l, LSX)];
          A = mk(zk.x + zm.x, zk.y - zm.y);
          B = mk(zk.y + zm.y, zm.x - zk.x);
        }
        if (wa) da[k] = A;
        if (wb) db[k] = B;
      }
    }
  }
  };
  if (want_ke) tail(std::true_type{});
  else tail(std::false_type{});
}
template <typename T, bool LES, int DEN, int LYZ>
__global__ void __launch_bounds__(FFS_MAXT) k_x_pass(Inst<T> I) {
  b_x_pass<T, LES, DEN, LYZ>(I, Blk::here());
}
template <typename T, int DEN, int LYZ>
__global__ void __launch_bounds__(FFS_MAXT) k_x_pass_diag(Inst<T> I) {
  b_x_pass<T, true, DEN, LYZ, 0, true>(I, Blk::here());
}

// The spectral barrier (hyperviscosity_types.jl:32-48): log(esp(|k|, i, p, 1/4)) with
// esp = 1 for |k| <= i, exp(-(|k| - i)^2 / (p^(1/4) - |k|^(1/4))) for |k| < p, 0 beyond.
__device__ __forceinline__ double barrier_f(double k, double i, double p) {
  const double a = fabs(k);
  const double e = a <= i ? 1.0 : (a < p ? exp(-((a - i) * (a - i)) / (pow(p, 0.25) - pow(a, 0.25))) : 0.0);
  return log(e);
}
// the barrier as a stats / spectrum weight: -inf (beyond endk) counts 0 (stats.jl:1160-1161)
__device__ __forceinline__ double barrier_w(double k2, double i, double p) {
  const double f = barrier_f(sqrt(k2), i, p);
  return isinf(f) ? 0.0 : f;
}

// velocity integrating-factor exponent c(k^2) = -nu k^2 - nuh (k^2)^M (ETD.jl:60-95), or
// muladd(k^2, -nu, f(|k|)) with the spectral barrier f (ETD.jl:71-82); muladd is a
// single-rounding fma in the reference.
template <typename T> __device__ __forceinline__ double c_vel(const Inst<T>& I, double k2) {
  if (!I.hv) return dd::M(k2, -I.nu);
  if (I.hv_kind == 1) {
    // f = log(0) = -inf (beyond endk, or exp underflow): muladd gives -inf, whose ETD
    // coefficients are 0 (ETD.jl:182-191)
    const double f = barrier_f(sqrt(k2), I.hv_initk, I.hv_endk);
    return isinf(f) ? -INFINITY : dd::fma_e(k2, -I.nu, f);
  }
  double km = k2;
  for (int m = 1; m < I.hv_m; ++m) km = dd::M(km, k2);
  return dd::fma_e(k2, -I.nu, dd::M(km, -I.hv_nu));
}

// k^2 as the reference forms it: muladd(KX,KX, muladd(KY,KY, KZ*KZ)) with K = i / L
template <typename T> __device__ __forceinline__ double ref_k2(const Inst<T>& I, int ix, int iy, int iz) {
  const double kx = dd::D((double)ix, I.lx), ky = dd::D((double)iy, I.ly), kz = dd::D((double)iz, I.lz);
  return dd::fma_e(kx, kx, dd::fma_e(ky, ky, dd::M(kz, kz)));
}

// ====================================================================================
// Scalar kernel: set_dt! (time_step_functions.jl:86-129), integrator dt history
// (Adams_Bashforth.jl:37-47, ETD.jl:110-114), AB3 coefficients (Adams_Bashforth.jl
// 49-89), forcing energy of the band. mode 0: a step; mode 1: initialize!; mode 2: the
// run's tail (set_dt! and the forcing of calculate_rhs!, no integrator call).
// One CTA.
// ====================================================================================
template <typename T>
__device__ __forceinline__ void b_scalar(const Inst<T>& I, int mode, const Blk bk) {
  DevState* Sg = I.st;
  __shared__ double sh_ef[256];
  __shared__ double sh_dt;
  if (threadIdx.x == 0) {
    DevState S = *Sg;   // one load; all logic on the local copy
    const long long it = S.iteration;
    if (I.adaptive) {
      const double m = __longlong_as_double((long long)S.umax_bits);
      S.slot_u = I.ref_slot ? fmax(m, S.slot_u) : m;
      if (I.density) {
        const double mr = __longlong_as_double((long long)S.rhomax_bits);
        S.slot_rho = I.ref_slot ? fmax(mr, S.slot_rho) : mr;
      }
      const double umax = S.slot_u;
      const double dx = 2.0 * M_PI * I.ly / I.ny;
      double cfl = I.cfl;
      if (it == 0) cfl *= 0.1;
      else if (it == 1) cfl *= 0.2;
      else if (it == 2) cfl *= 0.4;
      else if (it == 3) cfl *= 0.8;
      double newdt = dd::D(dd::M(cfl, dx), umax);
      if (I.density && !I.scalar) {   // buoyancy cap (the passive scalar has none)
        const double den = dd::M(S.slot_rho, fabs(I.gval));
        newdt = fmin(newdt, dd::M(cfl, sqrt(dd::D(dx, den))));
      }
      if (it > 3) {
        const double dt = S.dt;
        newdt = newdt < dt ? fmax(dd::D(dt, 1.25), newdt) : fmin(dd::M(1.25, dt), newdt);
      }
      if (I.ab3 && !I.euler) {
        if (S.ts_iter == 0) { S.dt3 = S.dt2 = S.dt = dd::D(newdt, 2.0); }
        else { S.dt3 = S.dt2; S.dt2 = S.dt; S.dt = newdt; }
      } else {
        S.dt3 = S.dt2; S.dt2 = S.dt; S.dt = newdt;
      }
    }
    if (mode == 1) {
      // initialize! of the integrator: dt history := current dt (Adams_Bashforth.jl:28-35, ETD.jl:99-108)
      S.dt2 = S.dt; S.dt3 = S.dt;
      S.stage = 0;
      S.skip_table = 0;
    } else if (mode == 0) {
      const int prev_stage = S.stage;
      S.ts_iter += 1;
      const long long i = S.ts_iter;
      S.stage = i >= 3 ? 3 : (int)i;
      // with a fixed dt the stage-3 coefficients never change once computed
      S.skip_table = (!I.adaptive && prev_stage == 3 && S.stage == 3) ? 1 : 0;
      if (I.euler) {   // muladd(dt, rhs, u) (Euller.jl:14-25)
        S.At = S.dt; S.Bt = 0.0; S.Ct = 0.0;
      } else if (I.ab3) {
        const double dt = S.dt, dt2 = S.dt2, dt3 = S.dt3;
        if (I.adaptive) {
          S.At = (1. + (dt * (2 * dt + 6 * dt2 + 3 * dt3)) / (6 * dt2 * (dt2 + dt3))) * dt;
          S.Bt = (-dt * dt * (2 * dt + 3 * dt2 + 3 * dt3) / (6 * dt2 * dt3 * (dt + dt2))) * (dt + dt2);
          S.Ct = (dt * dt * (2 * dt + 3 * dt2) / (6 * dt3 * (dt + dt2 + dt3) * (dt2 + dt3))) * (dt + dt2 + dt3);
        } else {
          S.At = 23 * dt / 12; S.Bt = -16 * dt / 12; S.Ct = 5 * dt / 12;
        }
      }
    }
    *Sg = S;
    sh_dt = S.dt;
  }
  // isotropic band forcing: E_f = sum_{0<|k|<=kf} 1/2 w |u|^2 from the current u
  if (I.forcing && mode != 1) {
    const int bx = (int)floor(I.f_kf * I.lx) + 1, by = (int)floor(I.f_kf * I.ly) + 1, bz = (int)floor(I.f_kf * I.lz) + 1;
    const int cnt = bx * (2 * by + 1) * (2 * bz + 1);
    double e = 0.0;
    for (int t = threadIdx.x; t < cnt; t += blockDim.x) {
      const int ix = t % bx, r = t / bx, iy = r % (2 * by + 1) - by, iz = r / (2 * by + 1) - bz;
      if (ix >= I.Mx) continue;
      const double kx = ix / I.lx, ky = iy / I.ly, kz = iz / I.lz;
      const double k2 = kx * kx + ky * ky + kz * kz;
      if (k2 == 0.0 || k2 > I.f_kf * I.f_kf) continue;
      const int y = iy >= 0 ? iy : I.ny + iy, z = iz >= 0 ? iz : I.nz + iz;
      const int jc = ycomp(I, y), kc = zcomp(I, z);
      if (jc < 0 || kc < 0) continue;
      const long long idx = ((long long)kc * I.NYR + jc) * I.KXP + ix;
      double a = 0.0;
      for (int c = 0; c < 3; ++c) { cplx<T> v = I.uh[c * I.cstride + idx]; a += (double)v.x * v.x + (double)v.y * v.y; }
      e += 0.5 * (ix > 0 ? 2.0 : 1.0) * a;
    }
    // fixed-order reduction
    for (int o = 16; o > 0; o >>= 1) e += __shfl_xor_sync(0xffffffffu, e, o);
    if ((threadIdx.x & 31) == 0) sh_ef[threadIdx.x >> 5] = e;
    __syncthreads();
    if (threadIdx.x == 0) {
      double s = 0.0;
      for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += sh_ef[i];
      Sg->Ef = s;
      Sg->force_coef = s > 0.0 ? I.f_eps / (2.0 * s) : 0.0;
    }
  }
  // the update's scalars once here, so that no update thread does FP64 divisions
  if (threadIdx.x == 0) {
    const double dt = Sg->dt, dt2 = Sg->dt2, dt3 = Sg->dt3;
    const double c[5] = {Sg->At, Sg->Bt, Sg->Ct, -(dt3 + dt2) / dt2, dt * Sg->force_coef};
#pragma unroll
    for (int i = 0; i < 5; ++i) { Sg->coef_d[i] = c[i]; Sg->coef_f[i] = (float)c[i]; }
  }
}
template <typename T>
__global__ void k_scalar(Inst<T> I, int mode) {
  b_scalar<T>(I, mode, Blk::here());
}

// ====================================================================================
// kz = 0 plane forcing (rfForcing forcing.jl:6-114, cRfForcing cforcing.jl:1-97,
// nRfForcing nrforcing.jl, cNRfForcing cnrforcing.jl, aForcing aforcing.jl, QfForcing
// qfforcing.jl:1-81), from the current u after set_dt! (models.jl:6-9). One CTA, FP64.
// mode 1 (initialize!): the target spectrum Em of the initial field (forcing_types.jl
// :66-73; nRf/cNRf also N = Nm1 from the initial right-hand side; aForcing per mode);
// mode 0 / 2: the force of this step into pf_force and the powers hp, vp. Shell sums
// run one thread per shell over the shell's modes in a fixed order, the power sums
// through a fixed-order block reduction: every call is deterministic. nRf/cNRf read the
// step's right-hand side, so they run after the forward passes.
// ====================================================================================
// The projected right-hand side of a kz = 0 mode, as the update forms it
// (fourierspacep2!, models.jl:282-341): N + (AB3) explicit (hyper)viscosity + i k.tau
// + rho g, then the projection.
template <typename T>
__device__ __forceinline__ void plane_rhs(const Inst<T>& I, int m, double* out) {
  const long long cs = I.cstride;
  const int ix = m % I.KXP, jc = m / I.KXP;
  const int ky_i = ysig(I, jc);
  const T kx = kval(ix, I.Lx_t, I.iLx_t), ky = kval(ky_i, I.Ly_t, I.iLy_t), kz = T(0);
  const T k2 = kx * kx + (ky * ky + kz * kz);
  const bool k0 = ix == 0 && ky_i == 0;
  cplx<T> rhs[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) rhs[c] = I.sbuf[c * cs + m];
  if (I.ab3) {
    T cv;
    if (sizeof(T) == 8) {
      const double kd = (double)k2;
      double km = kd;
      for (int i = 1; i < I.hv_m; ++i) km = dd::M(km, kd);
      cv = T(I.hv ? dd::A(dd::M(kd, -I.nu), dd::M(km, -I.hv_nu)) : dd::M(kd, -I.nu));
    } else {
      cv = k2 * (-I.nu_t);
      if (I.hv) { T km = k2; for (int i = 1; i < I.hv_m; ++i) km *= k2; cv += km * (-I.hvnu_t); }
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) rhs[c] = rhs[c] + scl(I.uh[c * cs + m], cv);
  }
  if (I.les) {
#pragma unroll
    for (int c = 0; c < 3; ++c) rhs[c] = rhs[c] + I.sbuf[(4 + c) * cs + m];
  }
  if (I.density) rhs[I.gdir] = rhs[I.gdir] + scl(I.uh[3 * cs + m], I.gval_t);
  const cplx<T> kd = mk(kx * rhs[0].x + ky * rhs[1].x + kz * rhs[2].x, kx * rhs[0].y + ky * rhs[1].y + kz * rhs[2].y);
  const T inv = k0 ? T(0) : T(1) / k2;
  const cplx<T> p1 = mk(-kd.x * inv, -kd.y * inv);
  rhs[0] = rhs[0] + scl(p1, kx);
  rhs[1] = rhs[1] + scl(p1, ky);
  out[0] = rhs[0].x; out[1] = rhs[0].y; out[2] = rhs[1].x; out[3] = rhs[1].y;
}

template <typename T>
__global__ void __launch_bounds__(256) k_plane_forcing(Inst<T> I, int mode) {
  DevState* S = I.st;
  const int nsh = I.pf_nsh;
  double* R = I.pf_d;
  double* Em = R + nsh;
  double* fac = Em + nsh;
  const double* kh = fac + nsh;
  const double* Zf = kh + nsh;
  const double* QR = Zf + nsh;
  double* Nn = const_cast<double*>(QR) + nsh;
  double* Nm1 = Nn + nsh;
  const int kind = I.pforce;
  const bool qf = kind == FFS_PF_QF, af = kind == FFS_PF_A;
  const bool nl = kind == FFS_PF_NRF || kind == FFS_PF_CNRF;
  const long long cs = I.cstride;
  const int plane = I.NYR * I.KXP;
  double* EfS = Nm1 + nsh;         // Ef of the last forcing call (the Eh.N files)
  double* R2 = EfS + nsh;          // aForcing, per plane mode
  double* Em2 = R2 + plane;
  double* fac2 = Em2 + plane;
  const double* Zf2 = fac2 + plane;
  __shared__ double Ef[FFS_PF_MAXSH];
  __shared__ double NS[FFS_PF_MAXSH];
  __shared__ double red[2][256];
  const double nu = I.nu;
  auto modes_a2 = [&](int m) {
    const cplx<T> a = I.uh[m], b = I.uh[cs + m];
    return (double)a.x * a.x + (double)a.y * a.y + ((double)b.x * b.x + (double)b.y * b.y);
  };
  // calculate_u1u2_spectrum! / calculate_u1u2_mag_spectrum! (spectrum.jl:1-65) and, for
  // nRf/cNRf, calculate_nn_spectrum! (nrforcing.jl: proj(u, rhs - nu k^2 u) per shell)
  if (!af) {
    for (int n = threadIdx.x; n < nsh; n += blockDim.x) {
      double e = 0.0, en = 0.0;
      for (int q = I.pf_start[n]; q < I.pf_start[n + 1]; ++q) {
        const int m = I.pf_modes[q];
        const double cf = (m % I.KXP) > 0 ? 2.0 : 1.0;
        const double a2 = modes_a2(m);
        e += qf ? cf * sqrt(a2) : 0.5 * cf * a2;
        if (nl) {
          double r[4];
          plane_rhs<T>(I, m, r);
          const int ix = m % I.KXP;
          const double kx = ix / I.lx, ky = ysig(I, m / I.KXP) / I.ly;
          const double k2 = kx * kx + ky * ky;
          const double ax = I.uh[m].x, ay = I.uh[m].y, bx = I.uh[cs + m].x, by = I.uh[cs + m].y;
          const double nk = nu * k2;
          en += cf * (fma(ax, r[0] - nk * ax, ay * (r[1] - nk * ay)) + fma(bx, r[2] - nk * bx, by * (r[3] - nk * by)));
        }
      }
      Ef[n] = e;
      NS[n] = en;
    }
  }
  __syncthreads();
  const double eps = 2.220446049250313e-16;
  if (mode == 1) {
    if (af) {
      for (int m = threadIdx.x; m < plane; m += blockDim.x)
        Em2[m] = 0.5 * ((m % I.KXP) > 0 ? 2.0 : 1.0) * modes_a2(m);
    } else if (!qf) {
      for (int n = threadIdx.x; n < nsh; n += blockDim.x) {
        Em[n] = Ef[n];
        if (nl) { Nn[n] = NS[n]; Nm1[n] = NS[n]; }
      }
    }
    return;
  }
  if (!af)
    for (int n = threadIdx.x; n < nsh; n += blockDim.x) EfS[n] = Ef[n];
  const double dt = S->dt;
  const long long it = S->iteration;
  const double kf = I.pf_kf, alpha = I.pf_alpha;
  double omega = 0.0;
  if (kind == FFS_PF_RF || kind == FFS_PF_NRF) {   // ts = dt / cfl with the CFL ramp
    double ts = dt / I.pf_cfl;
    if (I.adaptive) {
      if (it == 0) ts /= 0.1;
      else if (it == 1) ts /= 0.2;
      else if (it == 2) ts /= 0.4;
      else if (it == 3) ts /= 0.8;
    }
    omega = (2 * M_PI) / (I.pf_tf * ts);
  } else if (kind == FFS_PF_CRF) {
    omega = (2 * M_PI) / I.pf_tf;                   // ts = Tf, omega = 2 pi / ts
  } else if (kind == FFS_PF_CNRF) {
    omega = (2 * M_PI) / (I.pf_tf * I.pf_tf);       // ts = Tf, omega = 2 pi / (Tf ts)
  } else if (af) {
    omega = (2 * M_PI) / (I.pf_tf * (10 * dt));     // ts = 10 dt
  }
  if (!qf && !af) {   // the shells' ODE (forcing.jl:47-53, nrforcing.jl)
    const double dtm2 = S->dt2;
    for (int n = 1 + threadIdx.x; n < nsh; n += blockDim.x) {
      if (nl) { Nm1[n] = Nn[n]; Nn[n] = NS[n]; }
      if (kh[n] <= kf) {
        double r;
        if (nl) r = R[n] + dt * (-2 * alpha * omega * (R[n] + Nn[n]) - (Nn[n] - Nm1[n]) / dtm2 -
                                 omega * omega * (Ef[n] - Em[n]));
        else r = R[n] + dt * (-2 * alpha * omega * R[n] - omega * omega * (Ef[n] - Em[n]));
        r = fmax(0.0, r);
        R[n] = r;
        fac[n] = sqrt(r / fmax(Ef[n], eps)) * Zf[n] * dt;
      }
    }
    if (nl && threadIdx.x == 0) { Nm1[0] = Nn[0]; Nn[0] = NS[0]; }
  }
  __syncthreads();
  // horizontal forcing of the kz = 0 plane (forcing.jl:57-77, aforcing.jl, qfforcing.jl:22-45)
  double ff = 0.0, fv = 0.0;
  for (int m = threadIdx.x; m < plane; m += blockDim.x) {
    const int n = I.pf_nmode[m];
    cplx<T> f1 = mk(T(0), T(0)), f2 = f1;
    if (n >= 0) {
      const cplx<T> a = I.uh[m], b = I.uh[cs + m];
      const double ax = a.x, ay = a.y, bx = b.x, by = b.y;
      const double cf = (m % I.KXP) > 0 ? 2.0 : 1.0;
      double s1x, s1y, s2x, s2y;
      if (qf) {
        const double umag = sqrt(ax * ax + ay * ay + (bx * bx + by * by));
        const double fkn = dt * QR[n] * 0.99 / Ef[n];
        s1x = (ax / umag) * fkn; s1y = (ay / umag) * fkn; s2x = (bx / umag) * fkn; s2y = (by / umag) * fkn;
        fv += (fma(ax, s1x / dt, ay * (s1y / dt)) + fma(bx, s2x / dt, by * (s2y / dt))) * cf;
      } else {
        double g;
        if (af) {   // the ODE of this mode (aforcing.jl)
          const double e = 0.5 * cf * (ax * ax + ay * ay + (bx * bx + by * by));
          const double r = fmax(0.0, R2[m] + dt * (-2 * alpha * omega * R2[m] - omega * omega * (e - Em2[m])));
          R2[m] = r;
          g = sqrt(r / fmax(e, eps)) * Zf2[m] * dt;
          fac2[m] = g;
        } else {
          g = fac[n];
        }
        s1x = ax * g; s1y = ay * g; s2x = bx * g; s2y = by * g;
        ff += (s1x * s1x + s1y * s1y + (s2x * s2x + s2y * s2y)) * cf;
        fv += (fma(ax, s1x, ay * s1y) + fma(bx, s2x, by * s2y)) * cf;
      }
      f1 = mk(T(s1x), T(s1y));
      f2 = mk(T(s2x), T(s2y));
    }
    I.pf_force[m] = f1;
    I.pf_force[plane + m] = f2;
  }
  red[0][threadIdx.x] = ff;
  red[1][threadIdx.x] = fv;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) { red[0][threadIdx.x] += red[0][threadIdx.x + o]; red[1][threadIdx.x] += red[1][threadIdx.x + o]; }
    __syncthreads();
  }
  if (threadIdx.x != 0) return;
  const double hp = qf ? red[1][0] : red[0][0] * 0.5 / dt + red[1][0] / dt;
  // vertical forcing of the (0, 0, kz) modes, kz = +-1..+-5 (Rf family) or +-3..+-5 (Qf)
  cplx<T>* fvert = I.pf_force + 2 * plane;
  auto at = [&](int kz) -> long long {   // compact index of (0, 0, kz)
    const int kc = kz >= 0 ? kz : I.NZR + kz;
    return (long long)kc * I.NYR * I.KXP;
  };
  double usum = 0.0;
  for (int k = 1; k <= 5; ++k)
    for (int sg = 1; sg >= -1; sg -= 2) {
      if (qf && k < 3) continue;
      const long long g = at(sg * k);
      const double a2 = (double)I.uh[g].x * I.uh[g].x + (double)I.uh[g].y * I.uh[g].y;
      const double b2 = (double)I.uh[cs + g].x * I.uh[cs + g].x + (double)I.uh[cs + g].y * I.uh[cs + g].y;
      usum += qf ? a2 + b2 : sqrt(a2 + b2);
    }
  const double f = qf ? dt * hp * (1 - 0.99) / (usum * 0.99) : dt * sqrt(2.0 * hp * (1.0 - 0.99)) / usum;
  double ffv = 0.0, fvv = 0.0;
  for (int k = 1; k <= 5; ++k)
    for (int sg = 1; sg >= -1; sg -= 2) {
      const int slot = (k - 1) + (sg > 0 ? 0 : 5);
      const bool on = !(qf && k < 3);
      const long long g = at(sg * k);
      const double ax = I.uh[g].x, ay = I.uh[g].y, bx = I.uh[cs + g].x, by = I.uh[cs + g].y;
      const double s1x = on ? ax * f : 0.0, s1y = on ? ay * f : 0.0, s2x = on ? bx * f : 0.0, s2y = on ? by * f : 0.0;
      fvert[slot] = mk(T(s1x), T(s1y));
      fvert[10 + slot] = mk(T(s2x), T(s2y));
      if (!on) continue;
      if (qf) {
        fvv += fma(ax, s1x / dt, ay * (s1y / dt)) + fma(bx, s2x / dt, by * (s2y / dt));
      } else {
        ffv += s1x * s1x + s1y * s1y + (s2x * s2x + s2y * s2y);
        fvv += fma(ax, s1x, ay * s1y) + fma(bx, s2x, by * s2y);
      }
    }
  S->pf_hp = hp;
  S->pf_vp = qf ? fvv : ffv * 0.5 / dt + fvv / dt;
}

// ETD coefficient tables for the current stage and dt history: by q = i^2 + j^2 + l^2
// when k^2 = q / L^2 is exact (uniform domain with L a power of two), else one entry per
// retained mode (compact index). Multi-CTA; runs after k_scalar.
template <typename T>
__device__ __forceinline__ void b_etd_table(const Inst<T>& I, int mode, const Blk bk) {
  const DevState* S = I.st;
  const int stage = S->stage;
  if (mode != 0 || stage == 0 || S->skip_table) return;
  const double dt = S->dt, dt2 = S->dt2, dt3 = S->dt3;
  const long long count = I.uniformL ? (long long)I.qmax + 1 : I.cstride;
  for (long long q = (long long)bk.x * blockDim.x + threadIdx.x; q < count; q += (long long)bk.nx * blockDim.x) {
    double k2;
    if (I.uniformL) {
      k2 = dd::D((double)q, I.lx * I.lx);
    } else {
      int ix, jc, kc;
      decomp(I, (unsigned)q, ix, jc, kc);
      if (ix >= I.Mx) continue;
      k2 = ref_k2(I, ix, ysig(I, jc), zsig(I, kc));
    }
    double E, A, B, C;
    etd_coeffs_exact<sizeof(T) == 8>(c_vel(I, k2), dt, dt2, dt3, stage, E, A, B, C);
    T* e = I.etab + 4 * q;
    e[0] = T(E); e[1] = T(A); e[2] = T(B); e[3] = T(C);
    if (I.density && I.etab_rho) {
      // c = -alpha k^2; the passive scalar's ETD3rdO takes the velocity's hyperviscosity
      // (simulationtypes.jl:336): muladd(k2, -alpha, k2^M * -nuh) or with the barrier
      // muladd(k2, -alpha, f(|k|)); the density its own (densityHyperViscosity,
      // density_stratification_types.jl:137-148, 172-176)
      double cr = dd::M(k2, -I.alpha);
      const int hk = I.scalar ? (I.hv ? (I.hv_kind == 1 ? 2 : 1) : 0) : I.rho_hv;
      if (hk == 1) {
        const int M = I.scalar ? I.hv_m : I.rho_hv_m;
        double km = k2;
        for (int m = 1; m < M; ++m) km = dd::M(km, k2);
        cr = dd::fma_e(k2, -I.alpha, dd::M(km, -(I.scalar ? I.hv_nu : I.rho_hv_nu)));
      } else if (hk == 2) {
        const double f = barrier_f(sqrt(k2), I.scalar ? I.hv_initk : I.rho_hv_initk, I.scalar ? I.hv_endk : I.rho_hv_endk);
        cr = isinf(f) ? -INFINITY : dd::fma_e(k2, -I.alpha, f);
      }
      etd_coeffs_exact<sizeof(T) == 8>(cr, dt, dt2, dt3, stage, E, A, B, C);
      T* r = I.etab_rho + 4 * q;
      r[0] = T(E); r[1] = T(A); r[2] = T(B); r[3] = T(C);
    }
  }
}
template <typename T>
__global__ void k_etd_table(Inst<T> I, int mode) {
  b_etd_table<T>(I, mode, Blk::here());
}

// ====================================================================================
// Forward z pass (myfourier! z-part + dealias + 1/N + rhs[1]=0, models.jl:171-175):
// the three components of N = FFT(u x w) together, plus the auxiliary fields (kinetic
// energy at stats/spectrum iterations; i k . tau for LES, models.jl:328-332; i k . flux
// for density, vectorfunctions.jl:93-103). Retained modes only, written compactly to
// the scratch buffer: [N(3)][ke][i k.tau(3)][i k.flux].
// grid (KXP/TX, NYR); block 3 TX tpl_z.
// ====================================================================================
template <typename T, int TX, int N = 0, bool SEQ = false>
__device__ __forceinline__ void b_fwd_z(const Inst<T>& I, const FieldList& F, int mode, const Blk bk) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int L3 = 3 * TX;
  constexpr int LB = SEQ ? TX : L3;   // lines held at once: one component (SEQ) or all three
  const int nz = I.nz, NZR = I.NZR;
  cplx<T>* buf = reinterpret_cast<cplx<T>*>(smem_raw);   // [srows(nz)][LB]
  cplx<T>* bufB = buf + srows(nz) * LB;                  // second buffer (plans of >= 3 passes)
  cplx<T>* accT = bufB + (I.pz.np >= 3 ? srows(nz) * LB : 0);   // [3][NZR][TX] i k . tau (LES)
  cplx<T>* accF = accT + 3 * NZR * TX;                   // [NZR][TX]    i k . flux (density)

  const long long it = I.st->iteration;
  const bool want_ke = ((it % I.dt_stat) == 0) || (mode != 1 && (it % I.dt_spec) == 0);
  const int kx0 = bk.x * TX, jc = bk.y;
  const int rowstride = I.NYR * I.KXP;
  const long long cs = I.cstride;
  const T kyv = kval(ysig(I, jc), I.Ly_t, I.iLy_t);
  const T Lx = I.Lx_t, iLx = I.iLx_t, Lz = I.Lz_t, iLz = I.iLz_t;
  const T sc = I.inv_n2_t;   // 1/N and the 1/2 the x pass's Hermitian unpack leaves out
  cplx<T>* out = I.sbuf + (long long)jc * I.KXP + kx0;   // + kc * rowstride + l (+ slot * cs)
  const bool aux = I.les || I.density;

  if (aux) {
    for (int e = threadIdx.x; e < 4 * NZR * TX; e += blockDim.x) accT[e] = mk(T(0), T(0));
    __syncthreads();
  }
  // auxiliary fields one at a time (TX lines each)
  int ns0 = 0, ns1 = 1, ns2 = 2;   // slots of N (scalars: no local-memory array)
  for (int fi = 0; fi < F.n; ++fi) {
    const int role = F.code[fi];
    if (role <= R_NZ) {
      if (role == R_NX) ns0 = F.slot[fi];
      else if (role == R_NY) ns1 = F.slot[fi];
      else ns2 = F.slot[fi];
      continue;
    }
    if (role == R_KE && !want_ke) continue;
    const cplx<T>* in = I.wz + (long long)F.slot[fi] * I.wzs + (long long)jc * I.KXP + kx0;
    auto ld = [&](int l, int z) -> cplx<T> { return in[(long long)z * rowstride + l]; };
    auto st = [&](int l, int z, cplx<T> v) {
      const int kc = zcomp(I, z);
      if (kc < 0) return;
      if (role == R_KE) { out[3 * cs + (long long)kc * rowstride + l] = scl(v, sc); return; }
      const int m = kc * TX + l;
      const T kx = kval(kx0 + l, Lx, iLx), ky = kyv, kz = kval(zsig(I, kc), Lz, iLz);
      // i k . tau for the traceless symmetric tau (models.jl:330); zz = -xx - yy
      auto addT = [&](int c, T kk, cplx<T> a) { cplx<T>& d = accT[c * NZR * TX + m]; d.x -= kk * a.y; d.y += kk * a.x; };
      switch (role) {
        case R_TXX: addT(0, kx, v); addT(2, -kz, v); break;
        case R_TXY: addT(0, ky, v); addT(1, kx, v); break;
        case R_TXZ: addT(0, kz, v); addT(2, kx, v); break;
        case R_TYY: addT(1, ky, v); addT(2, -kz, v); break;
        case R_TYZ: addT(1, kz, v); addT(2, ky, v); break;
        case R_FX: { cplx<T>& d = accF[m]; d.x -= kx * v.y; d.y += kx * v.x; } break;
        case R_FY: { cplx<T>& d = accF[m]; d.x -= ky * v.y; d.y += ky * v.x; } break;
        default: { cplx<T>& d = accF[m]; d.x -= kz * v.y; d.y += kz * v.x; } break;
      }
    };
    fft_lines<-1, TX, T>(I.pz, buf, bufB, TX, I.twz, ld, st);
  }
  if constexpr (SEQ) {   // large nz: one component at a time (TX lines), straight to the scratch buffer
    const bool kzero_col = (kx0 == 0) && (ysig(I, jc) == 0);
#pragma unroll 1
    for (int c = 0; c < 3; ++c) {
      const int sl = c == 0 ? ns0 : (c == 1 ? ns1 : ns2);
      const cplx<T>* in = I.wz + (long long)sl * I.wzs + (long long)jc * I.KXP + kx0;
      auto ld = [&](int l, int z) -> cplx<T> { return in[(long long)z * rowstride + l]; };
      auto st = [&](int l, int z, cplx<T> v) {
        const int kc = zcomp(I, z);
        if (kc < 0) return;
        const bool k0 = kzero_col && l == 0 && z == 0;   // rhs.c[1] = 0 (models.jl:174)
        out[c * cs + (long long)kc * rowstride + l] = k0 ? mk(T(0), T(0)) : scl(v, sc);
      };
      fft_lines_n<-1, TX, T, N>(I.pz, buf, bufB, TX, I.twz, ld, st);
    }
  } else {   // the three components of N together (3 TX lines), straight to the scratch buffer
    const cplx<T>* in0 = I.wz + (long long)ns0 * I.wzs + (long long)jc * I.KXP + kx0;
    const cplx<T>* in1 = I.wz + (long long)ns1 * I.wzs + (long long)jc * I.KXP + kx0;
    const cplx<T>* in2 = I.wz + (long long)ns2 * I.wzs + (long long)jc * I.KXP + kx0;
    const bool kzero_col = (kx0 == 0) && (ysig(I, jc) == 0);
    auto ld = [&](int l, int z) -> cplx<T> {
      const int c = l / TX, x = l % TX;
      const cplx<T>* in = c == 0 ? in0 : (c == 1 ? in1 : in2);
      return in[(long long)z * rowstride + x];
    };
    auto st = [&](int l, int z, cplx<T> v) {
      const int kc = zcomp(I, z);
      if (kc < 0) return;
      const int c = l / TX, x = l % TX;
      const bool k0 = kzero_col && x == 0 && z == 0;   // rhs.c[1] = 0 (models.jl:174)
      out[c * cs + (long long)kc * rowstride + x] = k0 ? mk(T(0), T(0)) : scl(v, sc);
    };
    fft_lines_n<-1, L3, T, N>(I.pz, buf, bufB, L3, I.twz, ld, st);
  }
  if (aux) {
    for (int m = threadIdx.x; m < NZR * TX; m += blockDim.x) {
      const int l = m % TX, kc = m / TX;
      const long long o = (long long)kc * rowstride + l;
      if (I.les) {
#pragma unroll
        for (int c = 0; c < 3; ++c) out[(4 + c) * cs + o] = scl(accT[c * NZR * TX + m], sc);
      }
      if (I.density) out[7 * cs + o] = scl(accF[m], sc);
    }
  }
}
template <typename T, int TX, int N = 0, bool SEQ = false>
__global__ void __launch_bounds__(FFS_MAXT) k_fwd_z(Inst<T> I, FieldList F, int mode) {
  b_fwd_z<T, TX, N, SEQ>(I, F, mode, Blk::here());
}

// ====================================================================================
// Update (fourierspacep2!, models.jl:282-364; time_step!, models.jl:468-472 and
// time_step_functions.jl:72-80): rhs = N (+ explicit (hyper)viscosity for AB3) + i k.tau
// + rho g, projected; integrator (AB3 / ETD1-2-3); forcing increment; projection.
// Density: rho rhs = i k.flux - drho/dz u_g, own integrator. Flat over the retained modes.
// mode 1 (initialize!): fm1 = fm2 = rhs, no update.
// ====================================================================================
template <typename T>
__device__ __forceinline__ void b_update(const Inst<T>& I, int mode, const Blk bk) {
  const DevState* S = I.st;
  const long long cs = I.cstride;
  const int par = S->hist_parity;
  cplx<T>* __restrict__ hA = I.hist + (long long)par * I.ncomp * cs;         // fm1
  cplx<T>* __restrict__ hB = I.hist + (long long)(1 - par) * I.ncomp * cs;   // fm2 -> receives the new rhs
  cplx<T>* __restrict__ uh = I.uh;
  const cplx<T>* __restrict__ sb = I.sbuf;
  const int stage = S->stage;
  const T At = step_coef<T>(S, CO_A), Bt = step_coef<T>(S, CO_B), Ct = step_coef<T>(S, CO_C);
  const T fdt = step_coef<T>(S, CO_FDT);
  const T fix2 = step_coef<T>(S, CO_FIX2);
  const T Lx = I.Lx_t, iLx = I.iLx_t, Ly = I.Ly_t, iLy = I.iLy_t, Lz = I.Lz_t, iLz = I.iLz_t;
  bool bad = false;
  for (unsigned g = bk.x * blockDim.x + threadIdx.x; g < (unsigned)cs; g += bk.nx * blockDim.x) {
    int ix, jc, kc;
    decomp(I, g, ix, jc, kc);
    if (ix >= I.Mx) {   // padding columns stay zero
      if (mode == 0) for (int c = 0; c < I.ncomp; ++c) uh[c * cs + g] = mk(T(0), T(0));
      continue;
    }
    const int ky_i = ysig(I, jc), kz_i = zsig(I, kc);
    const T kx = kval(ix, Lx, iLx), ky = kval(ky_i, Ly, iLy), kz = kval(kz_i, Lz, iLz);
    const T k2 = kx * kx + (ky * ky + kz * kz);
    const bool k0 = (ix == 0) && (ky_i == 0) && (kz_i == 0);
    cplx<T> rhs[3], u[3], f1[3], f2[3];
    // every load of the mode first (history too), so that they are all in flight at once
#pragma unroll
    for (int c = 0; c < 3; ++c) { rhs[c] = sb[c * cs + g]; u[c] = uh[c * cs + g]; }
    if (mode == 0) {
#pragma unroll
      for (int c = 0; c < 3; ++c) { f1[c] = hA[c * cs + g]; f2[c] = hB[c * cs + g]; }
    }
    cplx<T> rho = mk(T(0), T(0));
    if (I.density) rho = uh[3 * cs + g];
    if (I.ab3) {   // explicit (hyper)viscosity, models.jl:320-326
      T cv;
      if (sizeof(T) == 8) {   // K2*m_nu + (K2^M)*m_nuh as written in models.jl:322
        const double kd = (double)k2;
        double km = kd;
        for (int i = 1; i < I.hv_m; ++i) km = dd::M(km, kd);
        cv = T(I.hv ? dd::A(dd::M(kd, -I.nu), dd::M(km, -I.hv_nu)) : dd::M(kd, -I.nu));
      } else {
        cv = k2 * (-I.nu_t);
        if (I.hv) { T km = k2; for (int i = 1; i < I.hv_m; ++i) km *= k2; cv += km * (-I.hvnu_t); }
      }
#pragma unroll
      for (int c = 0; c < 3; ++c) rhs[c] = rhs[c] + scl(u[c], cv);
    }
    if (I.les) {   // + i k . tau (models.jl:328-332)
#pragma unroll
      for (int c = 0; c < 3; ++c) rhs[c] = rhs[c] + sb[(4 + c) * cs + g];
    }
    if (I.density) rhs[I.gdir] = rhs[I.gdir] + scl(rho, I.gval_t);   // models.jl:334-336
    // 1/k^2 of both projections (one division: the FP64 pipe is the bound of the FP64 form)
    const T inv = k0 ? T(0) : T(1) / k2;
    {  // projection (models.jl:338-339)
      const cplx<T> kd = mk(kx * rhs[0].x + ky * rhs[1].x + kz * rhs[2].x, kx * rhs[0].y + ky * rhs[1].y + kz * rhs[2].y);
      const cplx<T> p1 = mk(-kd.x * inv, -kd.y * inv);
      rhs[0] = rhs[0] + scl(p1, kx); rhs[1] = rhs[1] + scl(p1, ky); rhs[2] = rhs[2] + scl(p1, kz);
    }
    // density rhs: i k . flux - drho/dz * u_g  (vectorfunctions.jl:93-103)
    cplx<T> rrhs = mk(T(0), T(0));
    if (I.density) {
      rrhs = sb[7 * cs + g] + scl(u[I.gdir], -I.dgrad_t);
      if (I.ab3) rrhs = rrhs + scl(rho, k2 * (-I.alpha_t));
    }
    if (mode == 1) {   // initialize!: fm1 = fm2 = rhs (Adams_Bashforth.jl:28-35, ETD.jl:99-108)
#pragma unroll
      for (int c = 0; c < 3; ++c) { hA[c * cs + g] = rhs[c]; hB[c * cs + g] = rhs[c]; }
      if (I.density) { hA[3 * cs + g] = rrhs; hB[3 * cs + g] = rrhs; }
      continue;
    }
    T E, A, B, C;
    const unsigned te = I.uniformL ? (unsigned)(ix * ix + ky_i * ky_i + kz_i * kz_i) : g;   // ETD table entry
    if (I.ab3) {
      E = T(1); A = At; B = Bt; C = Ct;
    } else {
      const T* e = I.etab + 4 * te;
      E = e[0]; A = e[1]; B = e[2]; C = e[3];
    }
    const bool band = I.forcing && k2 > T(0) && k2 <= I.kf2_t;
    cplx<T> un[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      if (I.ab3 && !I.euler && stage == 2) f2[c] = scl(rhs[c] - f1[c], fix2) + rhs[c];   // fix_fm2! (ETD.jl:130-140)
      // muladd(A, rhs, muladd(B, fm1, muladd(C, fm2, E u))); E = 1 for the explicit integrators
      if (I.ab3) un[c] = scl(rhs[c], A) + (scl(f1[c], B) + (scl(f2[c], C) + u[c]));
      else un[c] = scl(rhs[c], A) + (scl(f1[c], B) + (scl(f2[c], C) + scl(u[c], E)));
      if (band) un[c] = un[c] + scl(u[c], fdt);   // forcing increment (add_forcing!)
    }
    if (I.pforce) {   // add_Rf_forcing! (forcing_types.jl:54-64): the kz = 0 plane, then (0, 0, kz)
      const int plane = I.NYR * I.KXP;
      if (kz_i == 0) {
        un[0] = un[0] + I.pf_force[g];
        un[1] = un[1] + I.pf_force[plane + g];
      } else if (ix == 0 && ky_i == 0 && kz_i >= -5 && kz_i <= 5) {
        const int slot = kz_i > 0 ? kz_i - 1 : 4 - kz_i;
        un[0] = un[0] + I.pf_force[2 * plane + slot];
        un[1] = un[1] + I.pf_force[2 * plane + 10 + slot];
      }
    }
    {  // projection after the update (time_step_functions.jl:78)
      const cplx<T> kd = mk(kx * un[0].x + ky * un[1].x + kz * un[2].x, kx * un[0].y + ky * un[1].y + kz * un[2].y);
      const cplx<T> p1 = mk(-kd.x * inv, -kd.y * inv);
      un[0] = un[0] + scl(p1, kx); un[1] = un[1] + scl(p1, ky); un[2] = un[2] + scl(p1, kz);
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      bad |= !(isfinite(un[c].x) && isfinite(un[c].y));
      uh[c * cs + g] = un[c];
      hB[c * cs + g] = rhs[c];
    }
    if (I.density) {
      const cplx<T> r1 = hA[3 * cs + g];
      cplx<T> r2 = hB[3 * cs + g];
      if (I.ab3) {
        if (stage == 2 && !I.euler) r2 = scl(rrhs - r1, fix2) + rrhs;
        E = T(1); A = At; B = Bt; C = Ct;
      } else {
        const T* e = I.etab_rho + 4 * te;
        E = e[0]; A = e[1]; B = e[2]; C = e[3];
      }
      cplx<T> rn;
      if (I.ab3) rn = scl(rrhs, A) + (scl(r1, B) + (scl(r2, C) + rho));
      else rn = scl(rrhs, A) + (scl(r1, B) + (scl(r2, C) + scl(rho, E)));
      bad |= !(isfinite(rn.x) && isfinite(rn.y));
      uh[3 * cs + g] = rn;
      hB[3 * cs + g] = rrhs;
    }
  }
  if (mode == 0 && __syncthreads_or(bad) && threadIdx.x == 0) atomicOr(&I.st->err, 1u);
}
template <typename T>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 4 : 1) k_update(Inst<T> I, int mode) {
  b_update<T>(I, mode, Blk::here());
}

// calculate_specHV (spec.jl:424-450) of one mode's value ee into a field's H and V bins
// (FP64 atomics): the kx = 0 plane without the dk factors, as in the reference; bins
// past the ends are dropped (the reference writes them out of bounds).
template <typename T>
__device__ __forceinline__ void spec_bin(const Inst<T>& I, double* f, int stride, double ee, int ix, int nx, int nj,
                                         int nk) {
  double* H = f;
  double* V = f + stride;
  if (ix == 0) {
    if (nj < I.nbinH) { atomicAdd(&H[0], 0.5 * ee); atomicAdd(&H[nj], 0.5 * ee); }
    if (nk < I.nbinV) atomicAdd(&V[nk], ee);
  } else {
    const double e2 = 2.0 * ee;
    if (nx < I.nbinH) atomicAdd(&H[nx], 0.5 * e2 * I.maxdkh);
    if (nj < I.nbinH) atomicAdd(&H[nj], 0.5 * e2 * I.maxdkh);
    if (nk < I.nbinV) atomicAdd(&V[nk], e2 * I.dkz);
  }
}

// u spectrum of the current state on demand (ffs_spectrum): spectrum_u +
// calculate_specHV (spec.jl:316-327, 424-450) of the total energy 1/2 |u|^2, i.e. the
// reference's u.specH on the horizontal bins and u_h.specV + u_v.specV on the vertical
// ones. out: [stride] H then [stride] V, zeroed by the caller; FP64 bins.
template <typename T>
__global__ void k_spectrum_u(Inst<T> I, double* out, int stride) {
  const long long cs = I.cstride;
  const T Lx = I.Lx_t, iLx = I.iLx_t, Ly = I.Ly_t, iLy = I.iLy_t, Lz = I.Lz_t, iLz = I.iLz_t;
  for (unsigned g = blockIdx.x * blockDim.x + threadIdx.x; g < (unsigned)cs; g += gridDim.x * blockDim.x) {
    int ix, jc, kc;
    decomp(I, g, ix, jc, kc);
    if (ix >= I.Mx) continue;
    const T kx = kval(ix, Lx, iLx), ky = kval(ysig(I, jc), Ly, iLy), kz = kval(zsig(I, kc), Lz, iLz);
    double ee = 0.0;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const cplx<T> u = I.uh[c * cs + g];
      ee += (double)u.x * u.x + (double)u.y * u.y;
    }
    ee *= 0.5;
    const int nk = (int)rint(fabs((double)kz) / I.dkz), nj = (int)rint(fabs((double)ky) / I.maxdkh);
    const int nx = (int)rint(fabs((double)kx) / I.maxdkh);
    spec_bin(I, out, stride, ee, ix, nx, nj, nk);
  }
}

// ====================================================================================
// Stats and spectra of the state before the update: u from the spectral state, N, ke,
// i k.tau from the scratch buffer written by k_fwd_z (stats.jl:64-219,
// 289-307, 532-561, 608-705, 750-814, 897-980; spec.jl:316-327, 424-450;
// density_stratification_types.jl:192-211). Grid-stride over the retained modes, FP64
// accumulation, fixed-order per-CTA partials for k_finalize. Runs at stats/spectrum
// iterations only (returns at once otherwise).
// ====================================================================================
template <typename T>
__device__ __forceinline__ void b_stats(const Inst<T>& I, int mode, const Blk bk) {
  const DevState* S = I.st;
  const long long it = S->iteration;
  const bool stats_t = (it % I.dt_stat) == 0 || mode == 2;   // the run's tail always writes a row
  const bool spec_t = mode != 1 && (it % I.dt_spec) == 0;
  if (!stats_t && !spec_t) return;
  __shared__ double red[Q_COUNT][9];
  const long long cs = I.cstride;
  const cplx<T>* sb = I.sbuf;
  const cplx<T>* ub = I.uh;
  // per-mode products in T, per-thread sums in T over a few modes (the grid gives every
  // thread at most ~16 modes), FP64 from the warp reduction on
  const T fdt = step_coef<T>(S, CO_FDT);
  const T kf2 = I.kf2_t, gv = I.gval_t;
  const T Lx = I.Lx_t, iLx = I.iLx_t, Ly = I.Ly_t, iLy = I.iLy_t, Lz = I.Lz_t, iLz = I.iLz_t;
  const long long rec = S->nspec;
  const int stride = I.nbinH > I.nbinV ? I.nbinH : I.nbinV;
  double* sp = I.spec + rec * 2LL * I.nspecf * stride;
  T q[Q_COUNT];
#pragma unroll
  for (int i = 0; i < Q_COUNT; ++i) q[i] = T(0);
  for (unsigned g = bk.x * blockDim.x + threadIdx.x; g < (unsigned)cs; g += bk.nx * blockDim.x) {
    int ix, jc, kc;
    decomp(I, g, ix, jc, kc);
    if (ix >= I.Mx) continue;
    const int ky_i = ysig(I, jc), kz_i = zsig(I, kc);
    const T kx = kval(ix, Lx, iLx), ky = kval(ky_i, Ly, iLy), kz = kval(kz_i, Lz, iLz);
    const T k2 = kx * kx + (ky * ky + kz * kz);
    const T w = ix > 0 ? T(2) : T(1);
    const bool k0 = (ix == 0) && (ky_i == 0) && (kz_i == 0);
    cplx<T> u[3];
    T a2[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) { u[c] = ub[c * cs + g]; a2[c] = u[c].x * u[c].x + u[c].y * u[c].y; }
    if (spec_t && rec < I.spec_cap) {
      // spectrum_u + calculate_specHV (spec.jl:316-327, 424-450), FP64 bins
      const double hh = 0.5 * ((double)a2[0] + (double)a2[1]), vv = 0.5 * (double)a2[2];
      const int nk = (int)rint(fabs((double)kz) / I.dkz), nj = (int)rint(fabs((double)ky) / I.maxdkh);
      const int nx = (int)rint(fabs((double)kx) / I.maxdkh);
      spec_bin(I, sp + (2 * SF_U_H) * stride, stride, hh, ix, nx, nj, nk);
      spec_bin(I, sp + (2 * SF_U_V) * stride, stride, vv, ix, nx, nj, nk);
    }
    if (!stats_t) continue;
    // STAT_FIL weight Gaussfilter(SPEC_FIL_D2, k.k)^2 (utils.jl:220-225)
    T G2 = T(0);
    if (I.sfil) { const T G = exp(T(-I.fil_d2 / 24.0) * k2); G2 = G * G; }
    // velocity moments (velocity_stats, viscosity_stats, d*_squared_mean)
    if (k0) { q[Q_U1] += u[0].x; q[Q_U2] += u[1].x; q[Q_U3] += u[2].x; }
    q[Q_U12] += w * a2[0]; q[Q_U22] += w * a2[1]; q[Q_U32] += w * a2[2];
    q[Q_EH] += w * k2 * (a2[0] + a2[1]); q[Q_EV] += w * k2 * a2[2];
    if (I.sfil) {
      q[Q_FU12] += w * a2[0] * G2; q[Q_FU22] += w * a2[1] * G2; q[Q_FU32] += w * a2[2] * G2;
      q[Q_FEH] += w * k2 * (a2[0] + a2[1]) * G2; q[Q_FEV] += w * k2 * a2[2] * G2;
    }
    q[Q_D1DY] += w * ky * ky * a2[0]; q[Q_D1DX] += w * kx * kx * a2[0];
    q[Q_D2DY] += w * ky * ky * a2[1]; q[Q_D2DX] += w * kx * kx * a2[1];
    // non-linear transfer: (N - i k ke) . u (stats.jl:897-917)
    const cplx<T> ke = sb[3 * cs + g];
    const T kk[3] = {kx, ky, kz};
    T rx[3], ry[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const cplx<T> Nc = sb[c * cs + g];
      rx[c] = Nc.x + kk[c] * ke.y;
      ry[c] = Nc.y - kk[c] * ke.x;
    }
    {
      const T lh = w * (rx[0] * u[0].x + ry[0] * u[0].y + rx[1] * u[1].x + ry[1] * u[1].y);
      const T lv = w * (rx[2] * u[2].x + ry[2] * u[2].y);
      q[Q_NLH] += lh; q[Q_NLV] += lv;
      if (I.sfil) { q[Q_FNLH] += lh * G2; q[Q_FNLV] += lv * G2; }
    }
    // pressure transfer (stats.jl:764-814): rhs - i k ke (+ i k.tau + rho g), projected part
    if (I.les) {
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const cplx<T> dT = sb[(4 + c) * cs + g];
        rx[c] += dT.x; ry[c] += dT.y;
        const T pr = dT.x * u[c].x + dT.y * u[c].y;
        if (c < 2) q[Q_LESH] += w * pr; else q[Q_LESV] += w * pr;
        if (I.sfil) { if (c < 2) q[Q_FLESH] += w * pr * G2; else q[Q_FLESV] += w * pr * G2; }
      }
    }
    cplx<T> rho = mk(T(0), T(0));
    if (I.density) {
      rho = ub[3 * cs + g];
      rx[I.gdir] += rho.x * gv; ry[I.gdir] += rho.y * gv;
    }
    const T kdx = kx * rx[0] + ky * rx[1] + kz * rx[2];
    const T kdy = kx * ry[0] + ky * ry[1] + kz * ry[2];
    const T inv = k0 ? T(0) : T(1) / k2;
    const T p1x = -kdx * inv, p1y = -kdy * inv;
    {
      const T lh = w * (u[0].x * p1x * kx + u[0].y * p1y * kx + u[1].x * p1x * ky + u[1].y * p1y * ky);
      const T lv = w * (u[2].x * p1x * kz + u[2].y * p1y * kz);
      q[Q_PH] += lh; q[Q_PV] += lv;
      // STAT_FIL (stats.jl:880-885): the filtered terms land in the unfiltered sums
      if (I.sfil) { q[Q_PH] += lh * G2; q[Q_PV] += lv * G2; }
    }
    if (I.hv) {
      // (k^2)^M (hyperviscosity_stats, stats.jl:532-561) or the barrier weight f(|k|)
      // (spectral_barrier_stats, hyperviscosity_types.jl:51-82)
      T km = T(1);
      if (I.hv_kind == 1) km = T(barrier_w((double)k2, I.hv_initk, I.hv_endk));
      else for (int i = 0; i < I.hv_m; ++i) km *= k2;
      q[Q_HVH] += w * km * (a2[0] + a2[1]);
      q[Q_HVV] += w * km * a2[2];
      if (I.sfil) { q[Q_FHVH] += w * km * (a2[0] + a2[1]) * G2; q[Q_FHVV] += w * km * a2[2] * G2; }
    }
    if (I.forcing && mode != 1 && k2 > T(0) && k2 <= kf2) {
      q[Q_HP] += w * (fdt * (a2[0] + a2[1]) + T(0.5) * fdt * fdt * (a2[0] + a2[1]));
      q[Q_VP] += w * (fdt * a2[2] + T(0.5) * fdt * fdt * a2[2]);
    }
    if (I.density) {
      const T r2 = rho.x * rho.x + rho.y * rho.y;
      if (k0) q[Q_RHO] += rho.x;
      q[Q_RHO2] += w * r2;
      q[Q_DR1] += w * kx * kx * r2; q[Q_DR2] += w * ky * ky * r2; q[Q_DR3] += w * kz * kz * r2;
      q[Q_BF] += w * (u[I.gdir].x * rho.x + u[I.gdir].y * rho.y);
      T rw = T(0);
      if (I.rho_hv) {   // scalar_hvis_stats (stats.jl:1086-1110, 1145-1171)
        if (I.rho_hv == 2) rw = T(barrier_w((double)k2, I.rho_hv_initk, I.rho_hv_endk));
        else { rw = T(1); for (int i = 0; i < I.rho_hv_m; ++i) rw *= k2; }
        q[Q_RHV] += w * rw * r2;
      }
      if (I.rho_les && !I.scalar) {
        // scalar_les_stats (stats.jl:1032-1083): proj(i k . flux, rho), flux the whole
        // fourth-field flux (-rho u + the LES diffusion)
        const cplx<T> dF = sb[7 * cs + g];
        const T pr = w * (dF.x * rho.x + dF.y * rho.y);
        q[Q_RPR] += pr;
        if (I.sfil) q[Q_FRPR] += pr * G2;
      }
      if (I.sfil) {
        if (I.rho_hv) q[Q_FRHV] += w * rw * r2 * G2;
        q[Q_FRHO2] += w * r2 * G2;
        if (ix == I.Mx - 1) q[Q_FDR1] += w * kx * kx * r2 * G2;   // stats.jl:370 (ee_fil = ...)
        q[Q_FDR2] += w * ky * ky * r2 * G2; q[Q_FDR3] += w * kz * kz * r2 * G2;
        q[Q_FBF] += w * (u[I.gdir].x * rho.x + u[I.gdir].y * rho.y) * G2;
      }
    }
    // integral-length plane sums (stats.jl:952-980)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      if (ix == 0) q[Q_IL0 + 3 * c + 0] += a2[c];
      if (ky_i == 0) q[Q_IL0 + 3 * c + 1] += w * a2[c];
      if (kz_i == 0) q[Q_IL0 + 3 * c + 2] += w * a2[c];
    }
  }
  if (!stats_t) return;
  // fixed-order CTA reduction in FP64: warp shuffle tree, then warps in order
  const int wv = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
#pragma unroll
  for (int i = 0; i < Q_COUNT; ++i) {
    double v = (double)q[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) red[i][wv] = v;
  }
  __syncthreads();
  if (threadIdx.x < Q_COUNT) {
    double sum = 0.0;
    for (int i = 0; i < nw; ++i) sum += red[threadIdx.x][i];
    I.partials[(long long)bk.x * QPAD + threadIdx.x] = sum;
  }
}

// ====================================================================================
// The other write_spec spectra (spec.jl:1-146, 196-422) at spectrum iterations, from
// the same state as the stats (before the update): viscous 2 nu k^2 E(k), non-linear
// transfer proj(N - i k ke, u), pressure transfer proj(u, p k), LES proj(i k.tau, u),
// hyperviscous nuh k^2M |u|^2, and with density the buoyancy proj(u_z, g_z rho), rho,
// rho dissipation alpha k^2 |rho|^2 and rho transfer proj(i k.flux, rho). Each field is
// binned by calculate_specHV into H and V. Grid-stride over the retained modes.
// ====================================================================================
template <typename T>
__device__ __forceinline__ void b_spectra(const Inst<T>& I, int mode, const Blk bk) {
  const DevState* S = I.st;
  const long long it = S->iteration;
  if (!(mode != 1 && (it % I.dt_spec) == 0)) return;
  const long long rec = S->nspec;
  if (rec >= I.spec_cap) return;
  const long long cs = I.cstride;
  const cplx<T>* sb = I.sbuf;
  const cplx<T>* ub = I.uh;
  const int stride = I.nbinH > I.nbinV ? I.nbinH : I.nbinV;
  double* sp = I.spec + rec * 2LL * I.nspecf * stride;
  const T Lx = I.Lx_t, iLx = I.iLx_t, Ly = I.Ly_t, iLy = I.iLy_t, Lz = I.Lz_t, iLz = I.iLz_t;
  const double nu = I.nu, nuh = I.hv_nu, alpha = I.alpha;
  const double gz = (I.density && I.gdir == 2) ? I.gval : 0.0, gv = I.gval;
  for (unsigned g = bk.x * blockDim.x + threadIdx.x; g < (unsigned)cs; g += bk.nx * blockDim.x) {
    int ix, jc, kc;
    decomp(I, g, ix, jc, kc);
    if (ix >= I.Mx) continue;
    const int ky_i = ysig(I, jc), kz_i = zsig(I, kc);
    const T kx = kval(ix, Lx, iLx), ky = kval(ky_i, Ly, iLy), kz = kval(kz_i, Lz, iLz);
    const double k2 = (double)(kx * kx + (ky * ky + kz * kz));
    const bool k0 = (ix == 0) && (ky_i == 0) && (kz_i == 0);
    const int nk = (int)rint(fabs((double)kz) / I.dkz), nj = (int)rint(fabs((double)ky) / I.maxdkh);
    const int nx = (int)rint(fabs((double)kx) / I.maxdkh);
    auto bin = [&](int f, double v) { spec_bin(I, sp + (2 * f) * stride, stride, v, ix, nx, nj, nk); };
    cplx<T> u[3];
    double a2[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) { u[c] = ub[c * cs + g]; a2[c] = (double)u[c].x * u[c].x + (double)u[c].y * u[c].y; }
    // spectrum_viscosity of spectrum_u
    bin(SF_VIS_H, 2.0 * nu * k2 * (0.5 * (a2[0] + a2[1])));
    bin(SF_VIS_V, 2.0 * nu * k2 * (0.5 * a2[2]));
    // filter_spectrum! (spec.jl:452-472): the *_fil spectra after the unfiltered fields
    double G2 = 0.0;
    int ff = I.nspecf;
    if (I.sfil) {
      const double G = exp(-I.fil_d2 / 24.0 * k2);
      G2 = G * G;
      ff = I.nspecf - (I.pforce ? 1 : 0) - 8 - (I.hv ? 2 : 0) - ((I.density && !I.scalar) ? 4 : 0);
      bin(ff, G2 * (0.5 * (a2[0] + a2[1])));                  // u_fil_h, u_fil_v
      bin(ff + 1, G2 * (0.5 * a2[2]));
      bin(ff + 2, 2.0 * nu * k2 * (G2 * (0.5 * (a2[0] + a2[1]))));   // vis_fil of u_fil
      bin(ff + 3, 2.0 * nu * k2 * (G2 * (0.5 * a2[2])));
    }
    // spectrum_non_linear: proj(N - i k ke, u)
    const cplx<T> ke = sb[3 * cs + g];
    const T kk[3] = {kx, ky, kz};
    double rx[3], ry[3], nl[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const cplx<T> Nc = sb[c * cs + g];
      rx[c] = (double)Nc.x + (double)kk[c] * ke.y;
      ry[c] = (double)Nc.y - (double)kk[c] * ke.x;
      nl[c] = rx[c] * u[c].x + ry[c] * u[c].y;
    }
    bin(SF_NL_H, nl[0] + nl[1]);
    bin(SF_NL_V, nl[2]);
    if (I.sfil) { bin(ff + 4, G2 * (nl[0] + nl[1])); bin(ff + 5, G2 * nl[2]); }
    int f = SF_BASE_COUNT;
    double les[3] = {0, 0, 0};
    if (I.les) {
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const cplx<T> dT = sb[(4 + c) * cs + g];
        les[c] = (double)dT.x * u[c].x + (double)dT.y * u[c].y;
        rx[c] += dT.x; ry[c] += dT.y;
      }
    }
    cplx<T> rho = mk(T(0), T(0));
    if (I.density) {
      rho = ub[3 * cs + g];
      rx[I.gdir] += (double)rho.x * gv; ry[I.gdir] += (double)rho.y * gv;
    }
    {  // spectrum_pressure: p1 = -(k . rhs')/k^2, proj(u, p1 k)
      const double kdx = kx * rx[0] + ky * rx[1] + kz * rx[2];
      const double kdy = kx * ry[0] + ky * ry[1] + kz * ry[2];
      const double px = k0 ? 0.0 : -kdx / k2, py = k0 ? 0.0 : -kdy / k2;
      double pr[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) pr[c] = (double)u[c].x * (px * kk[c]) + (double)u[c].y * (py * kk[c]);
      bin(SF_PRESS_H, pr[0] + pr[1]);
      bin(SF_PRESS_V, pr[2]);
      if (I.sfil) { bin(ff + 6, G2 * (pr[0] + pr[1])); bin(ff + 7, G2 * pr[2]); }
    }
    if (I.les) { bin(f, les[0] + les[1]); bin(f + 1, les[2]); f += 2; }
    if (I.hv) {   // spectrum_hyperviscosity: nuh (k^2)^M proj(u, u); spectrum_spectral_barrier: f(|k|) proj(u, u)
      double km = k2;
      for (int i = 1; i < I.hv_m; ++i) km *= k2;
      if (I.hv_kind == 1) km = barrier_w(k2, I.hv_initk, I.hv_endk);
      const double nuh = I.hv_kind == 1 ? 1.0 : I.hv_nu;
      bin(f, nuh * km * (a2[0] + a2[1]));
      bin(f + 1, nuh * km * a2[2]);
      if (I.sfil) { bin(ff + 8, G2 * (nuh * km * (a2[0] + a2[1]))); bin(ff + 9, G2 * (nuh * km * a2[2])); }
      f += 2;
    }
    if (I.density && !I.scalar) {
      const double r2 = (double)rho.x * rho.x + (double)rho.y * rho.y;
      const cplx<T> dF = sb[7 * cs + g];
      bin(f, gz * ((double)u[2].x * rho.x + (double)u[2].y * rho.y));   // buoyancy_v
      bin(f + 1, r2);                                                     // rho
      bin(f + 2, alpha * k2 * r2);                                        // rhodiss
      bin(f + 3, (double)dF.x * rho.x + (double)dF.y * rho.y);           // rhonl
      if (I.sfil) {   // buoyancy_fil_v, rho_fil, rhodiss_fil (of the filtered rho, filtered again), rhonl_fil
        const int fd = ff + 8 + (I.hv ? 2 : 0);
        bin(fd, G2 * (gz * ((double)u[2].x * rho.x + (double)u[2].y * rho.y)));
        bin(fd + 1, G2 * r2);
        bin(fd + 2, G2 * (alpha * k2 * (G2 * r2)));
        bin(fd + 3, G2 * ((double)dF.x * rho.x + (double)dF.y * rho.y));
      }
    }
    if (I.pforce && mode == 0) {
      // write_spec_forcing (spec.jl:148-170, 262-271), after the step's forcing call
      // (models.jl:6-9): (proj(u1, f1) + proj(u2, f2)) / dt on the forced modes, the kz = 0
      // plane and the (0, 0, kz) modes; the run's tail writes none
      const int plane = I.NYR * I.KXP;
      cplx<T> f1 = mk(T(0), T(0)), f2 = f1;
      bool forced = false;
      if (kz_i == 0) {
        f1 = I.pf_force[g]; f2 = I.pf_force[plane + g]; forced = true;
      } else if (ix == 0 && ky_i == 0 && kz_i >= -5 && kz_i <= 5) {
        const int slot = kz_i > 0 ? kz_i - 1 : 4 - kz_i;
        f1 = I.pf_force[2 * plane + slot]; f2 = I.pf_force[2 * plane + 10 + slot]; forced = true;
      }
      if (forced)
        bin(I.nspecf - 1, ((double)u[0].x * f1.x + (double)u[0].y * f1.y +
                           ((double)u[1].x * f2.x + (double)u[1].y * f2.y)) / I.st->dt);
    }
  }
}
// stats and spectra in one launch: both return at once outside their iterations
template <typename T>
__global__ void __launch_bounds__(256) k_stats(Inst<T> I, int mode) {
  b_stats<T>(I, mode, Blk::here());
  b_spectra<T>(I, mode, Blk::here());
}

// ====================================================================================
// Finalize: stats record (stats.jl:64-219), reference reductionh reuse for the next
// CFL (time_step_functions.jl:87 with utils.jl:247-258), iteration/time advance
// (models.jl:14-15). One CTA of 1024 threads. mode 0: step, 1: initialize!, 2: the run's
// tail (writestats at the final iteration, FluidFlowSimulation.jl:46-49: a row whatever the
// iteration, non-linear and pressure columns from the last stats iteration unless this one
// is one, as s.nlstats/s.pressstats are; no iteration or time advance).
// ====================================================================================
template <typename T>
__device__ __forceinline__ void b_finalize(const Inst<T>& I, int mode, int nparts, const Blk bk) {
  DevState* S = I.st;
  __shared__ double tot[QPAD];
  const long long it = S->iteration;
  const bool fresh = (it % I.dt_stat) == 0;   // calculate_rhs! took the nl/pressure stats
  const bool stats_t = fresh || mode == 2;
  if (stats_t) {
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int qi = w; qi < Q_COUNT; qi += nw) {
      double s = 0.0;
      for (int c = lane; c < nparts; c += 32) s += I.partials[(long long)c * QPAD + qi];
      for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      if (lane == 0) tot[qi] = s;
    }
    __syncthreads();
  }
  if (threadIdx.x != 0) return;
  if (fresh) {
    S->nl_h = tot[Q_NLH]; S->nl_v = tot[Q_NLV];
    S->press_h = tot[Q_PH]; S->press_v = tot[Q_PV];
    if (I.sfil) {   // the filtered pressure sums are never accumulated (stats.jl:832-893)
      S->nl_hf = tot[Q_FNLH]; S->nl_vf = tot[Q_FNLV];
      S->press_hf = 0.0; S->press_vf = 0.0;
    }
  }
  if (mode == 1) {
    // calculate_rhs! at initialize!: pressure_stats leaves its sum in reductionh[1]
    if (stats_t && I.adaptive && I.ref_slot) S->slot_u = tot[Q_PH];
    S->umax_bits = 0ull; S->rhomax_bits = 0ull;
    return;
  }
  if (stats_t) {
    const long long r = S->nrec;
    if (r < I.rec_cap) {
      double* row = I.records + r * I.ncols;
      // the Stats.txt columns after iteration and time (stats.jl:64-165); f: the
      // Stats_fil.txt twin (filtered sums, the same means and forcing columns)
      auto stats_cols = [&](int c, bool f) -> int {
        const double u12 = tot[f ? Q_FU12 : Q_U12], u22 = tot[f ? Q_FU22 : Q_U22], u32 = tot[f ? Q_FU32 : Q_U32];
        const double kh = (u12 + u22) / 2, kv = u32 / 2;
        const double eh = I.nu * tot[f ? Q_FEH : Q_EH], ev = I.nu * tot[f ? Q_FEV : Q_EV];
        const double nlh = f ? S->nl_hf : S->nl_h, nlv = f ? S->nl_vf : S->nl_v;
        const double ph = f ? S->press_hf : S->press_h, pv = f ? S->press_vf : S->press_v;
        row[c++] = tot[Q_U1]; row[c++] = tot[Q_U2]; row[c++] = tot[Q_U3];
        row[c++] = u12; row[c++] = u22; row[c++] = u32;
        row[c++] = kh; row[c++] = kv; row[c++] = 2 * kv / kh; row[c++] = kh + kv;
        row[c++] = eh; row[c++] = ev; row[c++] = eh + ev;
        row[c++] = nlh; row[c++] = nlv; row[c++] = ph; row[c++] = pv;
        row[c++] = -(nlh + ph); row[c++] = nlv + pv;
        const double lesh = tot[f ? Q_FLESH : Q_LESH], lesv = tot[f ? Q_FLESV : Q_LESV];
        const double hvh = tot[f ? Q_FHVH : Q_HVH], hvv = tot[f ? Q_FHVV : Q_HVV];
        // hyperviscous columns: nuh x the (k^2)^M sums, or minus the barrier sums
        const double hvs = I.hv_kind == 1 ? -1.0 : I.hv_nu;
        double tdiss = eh + ev;
        if (I.les) tdiss += -lesh - lesv;
        if (I.hv) tdiss += hvs * (hvh + hvv);
        row[c++] = tdiss;
        if (I.density) {   // density (BoussinesqApproximation stats) or scalar_stats (stats.jl:221-233)
          const double d1 = tot[f ? Q_FDR1 : Q_DR1], d2 = tot[f ? Q_FDR2 : Q_DR2], d3 = tot[f ? Q_FDR3 : Q_DR3];
          const double rd = I.alpha * (d1 + d2 + d3);
          row[c++] = tot[Q_RHO]; row[c++] = tot[f ? Q_FRHO2 : Q_RHO2]; row[c++] = d1; row[c++] = d2;
          row[c++] = d3; row[c++] = rd;
          if (!I.scalar) {
            // density LES and hyperviscosity (density_stratification_types.jl:46-87):
            // trhodiss = rhodiss (+ rhopr) (+ rhohdiss), then bflux, rhopr, rhohdiss
            const double rpr = -tot[f ? Q_FRPR : Q_RPR];
            const double rh = I.rho_hv == 2 ? -tot[f ? Q_FRHV : Q_RHV] : I.rho_hv_nu * tot[f ? Q_FRHV : Q_RHV];
            double trd = rd;
            if (I.rho_les) trd += rpr;
            if (I.rho_hv) trd += rh;
            row[c++] = trd;
            row[c++] = -I.gval * tot[f ? Q_FBF : Q_BF];
            if (I.rho_les) row[c++] = rpr;
            if (I.rho_hv) row[c++] = rh;
          }
        }
        if (I.les) {
          const double prh = -lesh, prv = -lesv;
          row[c++] = prh; row[c++] = prv; row[c++] = (2 * prv) / prh; row[c++] = prh + prv;
        }
        if (I.forcing) {
          const double dt = S->dt;
          row[c++] = tot[Q_HP] / dt; row[c++] = tot[Q_VP] / dt; row[c++] = (tot[Q_HP] + tot[Q_VP]) / dt;
        } else if (I.pforce == FFS_PF_A) {   // stats(a::AForcing) (forcing_types.jl:98): hp, vp
          row[c++] = S->pf_hp; row[c++] = S->pf_vp;
        } else if (I.pforce) {   // stats(a::RfForcing) (forcing_types.jl:33): F.hp, F.vp of the last call
          row[c++] = S->pf_hp; row[c++] = S->pf_vp; row[c++] = S->pf_hp + S->pf_vp;
        }
        if (I.hv) {
          row[c++] = hvs * hvh; row[c++] = hvs * hvv; row[c++] = hvs * (hvh + hvv);
        }
        return c;
      };
      int c = 0;
      row[c++] = (double)it; row[c++] = S->time;
      c = stats_cols(c, false);
      // 9 integral-length plane sums and 4 derivative variances (Scales.txt inputs)
      for (int i = 0; i < 9; ++i) row[c++] = tot[Q_IL0 + i];
      row[c++] = tot[Q_D1DY]; row[c++] = tot[Q_D1DX]; row[c++] = tot[Q_D2DY]; row[c++] = tot[Q_D2DX];
      if (I.sfil) stats_cols(c, true);   // the Stats_fil.txt row (stats.jl:48-52)
    }
    S->nrec = r + 1;
    if (I.adaptive && I.ref_slot) {
      // the last reduction of writestats that reuses reductionh / density reduction
      double slot = tot[Q_D2DX];
      // STAT_FIL: the scalar's and the density's filtered sums go through reductionh
      // (scalar_stats, buoyancy_flux: density_stratification_types.jl:192-210)
      if (I.sfil && I.density)
        slot = I.scalar ? tot[Q_FDR3] : (I.rho_hv ? tot[Q_FRHV] : (I.rho_les ? tot[Q_FRPR] : tot[Q_FBF]));
      if (I.les) slot = tot[Q_LESH];
      if (I.hv) slot = tot[Q_HVH];
      S->slot_u = slot;
      // the density's reduction: the buoyancy flux sum, then its LES and hyperviscous sums
      if (I.density) S->slot_rho = I.rho_hv ? tot[Q_RHV] : ((I.rho_les && !I.scalar) ? tot[Q_RPR] : tot[Q_BF]);
    }
  }
  if (mode != 1 && (it % I.dt_spec) == 0) S->nspec += 1;
  if (mode == 2) { S->umax_bits = 0ull; S->rhomax_bits = 0ull; return; }
  S->iteration = it + 1;
  S->time += S->dt;
  S->hist_parity ^= 1;
  S->umax_bits = 0ull; S->rhomax_bits = 0ull;
}
template <typename T>
__global__ void __launch_bounds__(1024) k_finalize(Inst<T> I, int mode, int nparts) {
  b_finalize<T>(I, mode, nparts, Blk::here());
}

// ====================================================================================
// Transform-only helpers for set/get of physical fields (FP64 host layout
// [z][y][x], unpadded).
// ====================================================================================

// physical -> wy slots (r2c along x), nf fields paired two per complex line
template <typename T, int LIO = LYZ_IO>
__global__ void k_phys_fwd_x(Inst<T> I, int nf, int slot0) {
  constexpr int L = 2 * LIO;   // up to 4 fields -> 2 complex lines per (y,z)
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int n = I.nx;
  cplx<T>* s0 = reinterpret_cast<cplx<T>*>(smem_raw);   // [srows(n)][L+1]
  cplx<T>* s1 = s0 + srows(n) * (L + 1);
  cplx<T>* sx = fft_result_buffer(I.px, s0, s1);
  const int g0 = blockIdx.x * LIO;
  const long long plane = (long long)I.ny * I.nz * n;
  auto ld = [&](int l, int j) -> cplx<T> {
    const int p = l / LIO, q = l % LIO;
    const int fa = 2 * p, fb = 2 * p + 1;
    const long long base = (long long)(g0 + q) * n + j;
    const T a = fa < nf ? T(I.phys[fa * plane + base]) : T(0);
    const T b = fb < nf ? T(I.phys[fb * plane + base]) : T(0);
    return mk(a, b);
  };
  auto st = [&](int l, int j, cplx<T> v) { sx[sidx(j, l, L + 1)] = v; };
  fft_lines<-1, L, T>(I.px, s0, s1, L + 1, I.twx, ld, st);
  const int KXP = I.KXP;
  for (int e = threadIdx.x; e < L * KXP; e += blockDim.x) {
    const int k = e % KXP, l = e / KXP, p = l / LIO, q = l % LIO;
    cplx<T> A = mk(T(0), T(0)), B = mk(T(0), T(0));
    if (k < I.Mx) {
      const cplx<T> zk = sx[sidx(k, l, L + 1)];
      const cplx<T> zm = sx[sidx((n - k) % n, l, L + 1)];
      A = mk(T(0.5) * (zk.x + zm.x), T(0.5) * (zk.y - zm.y));
      B = mk(T(0.5) * (zk.y + zm.y), T(-0.5) * (zk.x - zm.x));
    }
    const long long off = (long long)(g0 + q) * KXP + k;
    if (2 * p < nf) I.wy[(long long)(slot0 + 2 * p) * I.wys + off] = A;
    if (2 * p + 1 < nf) I.wy[(long long)(slot0 + 2 * p + 1) * I.wys + off] = B;
  }
}

// wz slots -> compact spectral state: forward z, 1/N scaling, dealias (myfourier!)
template <typename T, int TX>
__global__ void __launch_bounds__(FFS_MAXT) k_fwd_z_store(Inst<T> I, FieldList F) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cplx<T>* s0 = reinterpret_cast<cplx<T>*>(smem_raw);
  cplx<T>* s1 = s0 + srows(I.nz) * TX;
  const int fi = blockIdx.x, kx0 = blockIdx.y * TX, jc = blockIdx.z;
  const int rowstride = I.NYR * I.KXP;
  const cplx<T>* in = I.wz + (long long)F.slot[fi] * I.wzs + (long long)jc * I.KXP + kx0;
  cplx<T>* out = I.uh + (long long)F.code[fi] * I.cstride + (long long)jc * I.KXP + kx0;
  const T sc = T(I.inv_n);
  auto ld = [&](int l, int z) -> cplx<T> { return in[(long long)z * rowstride + l]; };
  auto st = [&](int l, int z, cplx<T> v) {
    const int kc = zcomp(I, z);
    if (kc < 0) return;
    out[(long long)kc * rowstride + l] = (kx0 + l < I.Mx) ? scl(v, sc) : mk(T(0), T(0));
  };
  fft_lines<-1, TX, T>(I.pz, s0, s1, TX, I.twz, ld, st);
}

// wy slots -> physical (c2r along x) into the FP64 staging buffer
template <typename T, int LIO = LYZ_IO>
__global__ void k_inv_x_phys(Inst<T> I, int nf) {
  constexpr int L = 2 * LIO;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int n = I.nx, Mx = I.Mx;
  cplx<T>* s0 = reinterpret_cast<cplx<T>*>(smem_raw);
  cplx<T>* s1 = s0 + srows(n) * L;
  const int g0 = blockIdx.x * LIO;
  const long long plane = (long long)I.ny * I.nz * n;
  auto ld = [&](int l, int j) -> cplx<T> {
    const int p = l / LIO, q = l % LIO;
    const bool cj = 2 * j > n;
    const int k = cj ? n - j : j;
    if (k >= Mx) return mk(T(0), T(0));
    const int fa = 2 * p, fb = 2 * p + 1;
    const long long off = (long long)(g0 + q) * I.KXP + k;
    cplx<T> A = fa < nf ? I.wy[(long long)fa * I.wys + off] : mk(T(0), T(0));
    cplx<T> B = fb < nf ? I.wy[(long long)fb * I.wys + off] : mk(T(0), T(0));
    if (k == 0 || 2 * k == n) { A.y = T(0); B.y = T(0); }
    if (cj) { A.y = -A.y; B.y = -B.y; }
    return mk(A.x - B.y, A.y + B.x);
  };
  auto st = [&](int l, int j, cplx<T> v) {
    const int p = l / LIO, q = l % LIO;
    const long long base = (long long)(g0 + q) * n + j;
    if (2 * p < nf) I.phys[(2 * p) * plane + base] = (double)v.x;
    if (2 * p + 1 < nf) I.phys[(2 * p + 1) * plane + base] = (double)v.y;
  };
  fft_lines<+1, L, T>(I.px, s0, s1, L, I.twx, ld, st);
}

}  // namespace ffsgpu
