// Paired y/z passes (FP32, compile-time plans): the same passes as b_inv_z / b_inv_y /
// b_fwd_y / b_fwd_z in ffs_kernels.cuh, with the CTA's TX = 2 LP kx lines taken as LP
// pairs of adjacent lines. Each thread moves a pair with one 16-byte load or store and
// transforms it on the packed FP32 pipe (fft_lines_ct2), so a CTA needs LP * tpl threads
// and half the FP32 instructions of the one-line-per-thread form.
//
// Lines kx >= Mx inside a CTA read the spectrum's padding columns, which hold zeros
// (the update keeps them zero), and their transforms are zero like the one-line form's.
#pragma once
#include "ffs_kernels.cuh"

namespace ffsgpu {

constexpr int PAIR_LP = 4;   // pairs per CTA: the TX = 8 lines of the one-line form

// shared memory of a paired pass: one or two planes of N * LP 16-byte elements
template <int N, int LP> constexpr size_t pair_smem() {
  return (size_t)16 * N * LP * (CtPlan<N>::np >= 3 ? 2 : 1);
}

// ------------------------------------------------------------------------------------
// Inverse z pass with the spectral prologue (fourierspacep1!, models.jl:63-119).
// grid (nfields, KXP/TX, NYR); block LP * ct_tpl<N>()
// ------------------------------------------------------------------------------------
template <int N, int LP>
__device__ __forceinline__ void b_inv_z2(const Inst<float>& I, const FieldList& F, const Blk bk) {
  using T = float;
  constexpr int TX = 2 * LP;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cplx<float2>* s0 = reinterpret_cast<cplx<float2>*>(smem_raw);
  cplx<float2>* s1 = s0 + N * LP;
  const int fi = bk.x, kx0 = bk.y * TX, jc = bk.z;
  const int code = F.code[fi];
  const long long cs = I.cstride;
  const int rowstride = I.NYR * I.KXP;
  const int Mx = I.Mx;
  const cplx<T>* uh = I.uh + (long long)jc * I.KXP + kx0;
  const T kyv = kval(ysig(I, jc), I.Ly_t, I.iLy_t);
  const T iLx = I.iLx_t, Lz = I.Lz_t, iLz = I.iLz_t;
  int fam, ca = 0, cb = 0;
  switch (code) {
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
  // wavenumbers of axis d for both lines of pair lp at kc
  auto kax = [&](int d, int lp, int kc) -> float2 {
    if (d == 0) return make_float2(T(kx0 + 2 * lp) * iLx, T(kx0 + 2 * lp + 1) * iLx);
    const T k = d == 1 ? kyv : kval(zsig(I, kc), Lz, iLz);
    return make_float2(k, k);
  };
  cplx<T>* out = I.wz + (long long)F.slot[fi] * I.wzs + (long long)jc * I.KXP + kx0;
  auto st = [&](int lp, int z, cplx<float2> v) { st_pair(out + (long long)z * rowstride + 2 * lp, v); };
  if (fam == 0) {
    auto ld = [&](int lp, int z) -> cplx<float2> {
      const int kc = zcomp(I, z);
      if (kc < 0 || kx0 + 2 * lp >= Mx) return zero_pair();
      return ldg_pair(uh + oa + (long long)kc * rowstride + 2 * lp);
    };
    fft_lines_ct2<+1, LP, N>(s0, s1, I.twz, ld, st);
  } else if (fam == 1) {
    auto ld = [&](int lp, int z) -> cplx<float2> {   // i (k_b u_c - k_c u_b), (b, c) = (ca, cb)
      const int kc = zcomp(I, z);
      if (kc < 0 || kx0 + 2 * lp >= Mx) return zero_pair();
      const long long o = (long long)kc * rowstride + 2 * lp;
      const cplx<float2> ub = ldg_pair(uh + oa + o), uc = ldg_pair(uh + ob + o);
      const float2 kb = kax(ca, lp, kc), kc_ = kax(cb, lp, kc);
      return mk(kc_ * ub.y - kb * uc.y, kb * uc.x - kc_ * ub.x);
    };
    fft_lines_ct2<+1, LP, N>(s0, s1, I.twz, ld, st);
  } else {
    auto ld = [&](int lp, int z) -> cplx<float2> {   // (i/2)(k_a u_b + k_b u_a), (a, b) = (ca, cb)
      const int kc = zcomp(I, z);
      if (kc < 0 || kx0 + 2 * lp >= Mx) return zero_pair();
      const long long o = (long long)kc * rowstride + 2 * lp;
      const cplx<float2> ua = ldg_pair(uh + oa + o), ub = ldg_pair(uh + ob + o);
      const float2 ka = kax(ca, lp, kc), kb = kax(cb, lp, kc);
      const float2 h = make_float2(0.5f, 0.5f), nh = make_float2(-0.5f, -0.5f);
      const float2 qx = fma_(ka, ub.x, kb * ua.x), qy = fma_(ka, ub.y, kb * ua.y);
      return mk(nh * qy, h * qx);
    };
    fft_lines_ct2<+1, LP, N>(s0, s1, I.twz, ld, st);
  }
}
template <int N, int LP>
__global__ void __launch_bounds__(LP * ct_tpl<N>()) k_inv_z2(Inst<float> I, FieldList F) {
  b_inv_z2<N, LP>(I, F, Blk::here());
}

// ------------------------------------------------------------------------------------
// Inverse y pass: grid (nfields, KXP/TX, nz)
// ------------------------------------------------------------------------------------
template <int N, int LP>
__device__ __forceinline__ void b_inv_y2(const Inst<float>& I, const FieldList& F, const Blk bk) {
  using T = float;
  constexpr int TX = 2 * LP;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cplx<float2>* s0 = reinterpret_cast<cplx<float2>*>(smem_raw);
  cplx<float2>* s1 = s0 + N * LP;
  const int fi = bk.x, kx0 = bk.y * TX, z = bk.z;
  const int KXP = I.KXP;
  const cplx<T>* in = I.wz + (long long)F.slot[fi] * I.wzs + (long long)z * I.NYR * KXP + kx0;
  cplx<T>* out = I.wy + (long long)F.slot[fi] * I.wys + (long long)z * I.ny * KXP + kx0;
  auto ld = [&](int lp, int y) -> cplx<float2> {
    const int jc = ycomp(I, y);
    if (jc < 0) return zero_pair();
    return ldg_pair(in + (long long)jc * KXP + 2 * lp);
  };
  auto st = [&](int lp, int y, cplx<float2> v) { st_pair(out + (long long)y * KXP + 2 * lp, v); };
  fft_lines_ct2<+1, LP, N>(s0, s1, I.twy, ld, st);
}
template <int N, int LP>
__global__ void __launch_bounds__(LP * ct_tpl<N>()) k_inv_y2(Inst<float> I, FieldList F) {
  b_inv_y2<N, LP>(I, F, Blk::here());
}

// ------------------------------------------------------------------------------------
// Forward y pass (keeps retained ky only): grid (nfields, KXP/TX, nz)
// ------------------------------------------------------------------------------------
template <int N, int LP>
__device__ __forceinline__ void b_fwd_y2(const Inst<float>& I, const FieldList& F, const Blk bk) {
  using T = float;
  constexpr int TX = 2 * LP;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cplx<float2>* s0 = reinterpret_cast<cplx<float2>*>(smem_raw);
  cplx<float2>* s1 = s0 + N * LP;
  const int fi = bk.x, kx0 = bk.y * TX, z = bk.z;
  if (F.code[fi] == R_KE) {
    const long long it = I.st->iteration;
    if ((it % I.dt_stat) != 0 && (it % I.dt_spec) != 0) return;
  }
  const int KXP = I.KXP;
  const cplx<T>* in = I.wy + (long long)F.slot[fi] * I.wys + (long long)z * I.ny * KXP + kx0;
  cplx<T>* out = I.wz + (long long)F.slot[fi] * I.wzs + (long long)z * I.NYR * KXP + kx0;
  auto ld = [&](int lp, int y) -> cplx<float2> { return ldg_pair(in + (long long)y * KXP + 2 * lp); };
  auto st = [&](int lp, int y, cplx<float2> v) {
    const int jc = ycomp(I, y);
    if (jc >= 0) st_pair(out + (long long)jc * KXP + 2 * lp, v);
  };
  fft_lines_ct2<-1, LP, N>(s0, s1, I.twy, ld, st);
}
template <int N, int LP>
__global__ void __launch_bounds__(LP * ct_tpl<N>()) k_fwd_y2(Inst<float> I, FieldList F) {
  b_fwd_y2<N, LP>(I, F, Blk::here());
}

// ------------------------------------------------------------------------------------
// Forward z pass, one field at a time (the SEQ form of b_fwd_z): N (3 components) and,
// at stats/spectrum iterations, the kinetic energy, scaled by 1/n^3 and pruned to the
// retained kz, into the scratch spectrum. With LES / density the stress and flux fields
// are transformed the same way and accumulated as i k.tau and i k.flux (models.jl:330,
// density_stratification_types.jl) in shared memory, then written scaled.
// grid (KXP/TX, NYR); shared memory: the pair plane(s), then with LES / density
// [3][NZR][TX] i k.tau and [NZR][TX] i k.flux (fwd_z2_aux_bytes)
// ------------------------------------------------------------------------------------
template <int TX> size_t fwd_z2_aux_bytes(int NZR) { return sizeof(cplx<float>) * (size_t)4 * NZR * TX; }

template <int N, int LP>
__device__ __forceinline__ void b_fwd_z2(const Inst<float>& I, const FieldList& F, int mode, const Blk bk) {
  using T = float;
  constexpr int TX = 2 * LP;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cplx<float2>* s0 = reinterpret_cast<cplx<float2>*>(smem_raw);
  cplx<float2>* s1 = s0 + N * LP;
  cplx<T>* accT = reinterpret_cast<cplx<T>*>(s0 + (size_t)N * LP * (CtPlan<N>::np >= 3 ? 2 : 1));
  const int NZR = I.NZR;
  cplx<T>* accF = accT + 3 * NZR * TX;
  const long long it = I.st->iteration;
  const bool want_ke = ((it % I.dt_stat) == 0) || (mode != 1 && (it % I.dt_spec) == 0);
  const int kx0 = bk.x * TX, jc = bk.y;
  const int rowstride = I.NYR * I.KXP;
  const long long cs = I.cstride;
  const float2 sc = make_float2(I.inv_n2_t, I.inv_n2_t);   // 1/N and the x pass's unpack 1/2
  cplx<T>* out = I.sbuf + (long long)jc * I.KXP + kx0;   // + c * cs + kc * rowstride + l
  const bool kzero_col = (kx0 == 0) && (ysig(I, jc) == 0);
  const bool aux = I.les || I.density;
  if (aux) {
    for (int e = threadIdx.x; e < 4 * NZR * TX; e += blockDim.x) accT[e] = mk(T(0), T(0));
    __syncthreads();
  }
  const T iLx = I.iLx_t, Lz = I.Lz_t, iLz = I.iLz_t;
  const T kyv = kval(ysig(I, jc), I.Ly_t, I.iLy_t);
#pragma unroll 1
  for (int fi = 0; fi < F.n; ++fi) {
    const int role = F.code[fi];
    if (role == R_KE && !want_ke) continue;
    const cplx<T>* in = I.wz + (long long)F.slot[fi] * I.wzs + (long long)jc * I.KXP + kx0;
    auto ld = [&](int lp, int z) -> cplx<float2> { return ldg_pair(in + (long long)z * rowstride + 2 * lp); };
    if (role <= R_KE) {   // N components and the kinetic energy: scratch slots 0..3
      const int c = role;
      cplx<T>* o = out + (long long)c * cs;
      auto st = [&](int lp, int z, cplx<float2> v) {
        const int kc = zcomp(I, z);
        if (kc < 0) return;
        cplx<float2> r = mk(v.x * sc, v.y * sc);
        if (c < 3 && kzero_col && lp == 0 && z == 0) { r.x.x = 0.f; r.y.x = 0.f; }   // rhs.c[1] = 0 (models.jl:174)
        st_pair(o + (long long)kc * rowstride + 2 * lp, r);
      };
      fft_lines_ct2<-1, LP, N>(s0, s1, I.twz, ld, st);
    } else {   // stress / flux: accumulate i k . tau (traceless symmetric, zz = -xx - yy), i k . flux
      auto st = [&](int lp, int z, cplx<float2> v) {
        const int kc = zcomp(I, z);
        if (kc < 0) return;
        const int m = kc * TX + 2 * lp;
        const T kz = kval(zsig(I, kc), Lz, iLz);
        const T kxa = T(kx0 + 2 * lp) * iLx, kxb = T(kx0 + 2 * lp + 1) * iLx;
        // d += i k v for both lines of the pair (k per line)
        auto add = [&](cplx<T>* d, T ka, T kb) {
          d[0].x -= ka * v.y.x; d[0].y += ka * v.x.x;
          d[1].x -= kb * v.y.y; d[1].y += kb * v.x.y;
        };
        cplx<T>* t0 = accT + m;
        cplx<T>* t1 = accT + NZR * TX + m;
        cplx<T>* t2 = accT + 2 * NZR * TX + m;
        switch (role) {
          case R_TXX: add(t0, kxa, kxb); add(t2, -kz, -kz); break;
          case R_TXY: add(t0, kyv, kyv); add(t1, kxa, kxb); break;
          case R_TXZ: add(t0, kz, kz); add(t2, kxa, kxb); break;
          case R_TYY: add(t1, kyv, kyv); add(t2, -kz, -kz); break;
          case R_TYZ: add(t1, kz, kz); add(t2, kyv, kyv); break;
          case R_FX: add(accF + m, kxa, kxb); break;
          case R_FY: add(accF + m, kyv, kyv); break;
          default: add(accF + m, kz, kz); break;
        }
      };
      fft_lines_ct2<-1, LP, N>(s0, s1, I.twz, ld, st);
    }
  }
  if (aux) {
    for (int m = threadIdx.x; m < NZR * TX; m += blockDim.x) {
      const int l = m % TX, kc = m / TX;
      const long long o = (long long)kc * rowstride + l;
      if (I.les) {
#pragma unroll
        for (int c = 0; c < 3; ++c) out[(4 + c) * cs + o] = scl(accT[c * NZR * TX + m], I.inv_n2_t);
      }
      if (I.density) out[7 * cs + o] = scl(accF[m], I.inv_n2_t);
    }
  }
}
template <int N, int LP>
__global__ void __launch_bounds__(LP * ct_tpl<N>()) k_fwd_z2(Inst<float> I, FieldList F, int mode) {
  b_fwd_z2<N, LP>(I, F, mode, Blk::here());
}

}  // namespace ffsgpu
