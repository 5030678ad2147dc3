// Register-fused x pass for the Smagorinsky LES model (with or without Boussinesq
// density) in FP32 (realspace! + realspacecalculation! + calc_les! + find_max,
// models.jl:121-214, 228-280, les_real_calc.jl:13-139, utils.jl:247-258).
//
// Twelve real inputs u(3), w(3), S(5) (+ rho) ride as six complex lines, i.e. three
// packed pairs; twelve real outputs N(3), ke, tau(5) (+ flux(3)) as three pairs. Holding
// all twelve physical fields at R points per thread needs R = 8, so the x transform uses
// two different two-pass plans: inverse n = R0 * 8 (pass 0 radix R0 from the half
// spectra, pass 1 radix 8 into registers), forward n = 8 * R0 (pass 0 radix 8 from
// registers, pass 1 radix R0 in place). Thread (q, i) owns j = i + m n/8 of line q: the
// outputs of the inverse pass 1 and the inputs of the forward pass 0. So the last inverse
// pass, the products and the first forward pass run in registers:
//
//   global half spectra -> inverse pass 0 -> smem -> registers: inverse pass 1, products,
//   forward pass 0 -> smem -> forward pass 1 (in place) -> Hermitian unpack -> global
//
// The three pair planes hold one 16-byte cplx<float2> per (position, line), rows of the
// CTA's 8 lines with the line XOR-ed by (j ^ j>>3 ^ j>>4) & 7, which keeps every pass's
// quarter-warp accesses on 8 distinct bank groups for n = 64 and 128.
#pragma once
#include "ffs_xfused.cuh"

namespace ffsgpu {

template <int N> struct XLesCfg;
template <> struct XLesCfg<128> { static constexpr int R0 = 16, MINB = 4; };
template <> struct XLesCfg<64> { static constexpr int R0 = 8, MINB = 8; };

template <int N> struct XLes {
  static constexpr int R0 = XLesCfg<N>::R0;   // radix of inverse pass 0 / forward pass 1
  static constexpr int RR = 8;                // radix of the register passes
  static constexpr int LYZ = 8;               // (y,z) lines per CTA
  static constexpr int TPL = N / RR;          // threads per line in the register passes
  static constexpr int T0 = N / R0;           // butterflies per line in the radix-R0 passes
  static constexpr int NT = LYZ * TPL;
  static constexpr int PE = N * LYZ;          // 16-byte elements of one pair plane
  static size_t smem() { return (size_t)3 * PE * 16; }
  static __device__ __forceinline__ int pix(int j, int q) { return j * 8 + (q ^ ((j ^ (j >> 3) ^ (j >> 4)) & 7)); }
};

template <int N, bool DEN>
__device__ __forceinline__ void b_x_les(const Inst<float>& I, const Blk bk) {
  using T = float;
  using C = XLes<N>;
  constexpr int R0 = C::R0, RR = C::RR, LYZ = C::LYZ, TPL = C::TPL, T0 = C::T0, NT = C::NT, PE = C::PE;
  constexpr int NIN = DEN ? 12 : 11, NOUT = DEN ? 12 : 9;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cplx<float2>* P = reinterpret_cast<cplx<float2>*>(smem_raw);   // pair plane c at P + c * PE
  __shared__ T red[64];

  const int tid = threadIdx.x;
  const int q = tid / TPL, i = tid % TPL;
  const long long g0 = (long long)bk.x * LYZ;   // first (y,z) line of the CTA
  const int Mx = I.Mx, KXP = I.KXP;
  const long long it = I.st->iteration;
  const bool want_ke = ((it % I.dt_stat) == 0) || ((it % I.dt_spec) == 0);
  const cplx<float2>* __restrict__ twr = reinterpret_cast<const cplx<float2>*>(I.twx_r);

  // the input slabs of the CTA one resident wave ahead into L2 (as in the velocity-only
  // fused pass)
  if (I.x_pf_dist > 0 && tid < NIN) {
    const long long nb = (long long)bk.x + I.x_pf_dist;
    if (nb < (long long)I.ny * I.nz / LYZ)
      prefetch_l2(I.wy + (long long)tid * I.wys + nb * LYZ * KXP, (unsigned)(sizeof(cplx<T>) * LYZ * KXP));
  }

  // ---- inverse pass 0 (radix R0, p = 1): pair c carries lines (f0 + i f1, f2 + i f3) of
  // fields f = 4c .. 4c+3; Hermitian extension of the half spectra
#pragma unroll 1
  for (int b = tid; b < 3 * LYZ * T0; b += NT) {
    const int ii = b % T0, ql = (b / T0) % LYZ, c = b / (T0 * LYZ);
    const cplx<T>* F0 = I.wy + (long long)(4 * c) * I.wys + (g0 + ql) * KXP;
    const long long fs = I.wys;
    const bool f3 = 4 * c + 3 < NIN;   // the last input line's imaginary field exists
    cplx<float2> x[R0];
#pragma unroll
    for (int m = 0; m < R0; ++m) {
      int k;
      T sg;
      herm_index<N, R0>(ii, m, k, sg);
      cplx<T> a0 = mk(T(0), T(0)), b0 = a0, a1 = a0, b1 = a0;
      if (k < Mx) {
        a0 = ldg_c(F0 + k); b0 = ldg_c(F0 + fs + k); a1 = ldg_c(F0 + 2 * fs + k);
        if (f3) b1 = ldg_c(F0 + 3 * fs + k);
      }
      x[m] = mk(make_float2(fmaf(-sg, b0.y, a0.x), fmaf(-sg, b1.y, a1.x)),
                make_float2(fmaf(sg, a0.y, b0.x), fmaf(sg, a1.y, b1.x)));
    }
    dftR<R0, +1>(x);
#pragma unroll
    for (int m = 0; m < R0; ++m) P[c * PE + C::pix(ii * R0 + m, ql)] = x[m];
  }
  __syncthreads();

  // ---- inverse pass 1 (radix 8, p = R0) in registers: fields at j = i + TPL m
  T f[12][RR];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    cplx<float2> x[RR];
#pragma unroll
    for (int m = 0; m < RR; ++m) x[m] = P[c * PE + C::pix(i + TPL * m, q)];
#pragma unroll
    for (int m = 1; m < RR; ++m) { const cplx<float2> w = twr[m * TPL + i]; x[m] = twmul2<+1>(x[m], w.x, w.y); }
    dftR<RR, +1>(x);
#pragma unroll
    for (int m = 0; m < RR; ++m) {
      f[4 * c][m] = x[m].x.x; f[4 * c + 1][m] = x[m].y.x; f[4 * c + 2][m] = x[m].x.y; f[4 * c + 3][m] = x[m].y.y;
    }
  }
  __syncthreads();   // every thread has read the planes the forward pass 0 overwrites

  // ---- physical-space products (models.jl:224, 260, 266; les_real_calc.jl:77-79),
  // max |u| and |rho| (utils.jl:247-258), one output pair at a time, each followed by the
  // forward pass 0 (radix 8, no twiddles) of that pair
  T umax = T(0), rmax = T(0);
  const T les2 = T(2) * T(I.les_alpha);
  T nrm[RR];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    if (c == 1) {   // after u x w, when the vorticity registers are free
#pragma unroll
      for (int m = 0; m < RR; ++m) {   // tau = 2 c^2 D^2 |S| S with |S| = sqrt(S:S), S traceless
        const T xx = f[6][m], xy = f[7][m], xz = f[8][m], yy = f[9][m], yz = f[10][m];
        const T zz = -xx - yy;
        nrm[m] = les2 * sqrtf(xx * xx + yy * yy + zz * zz + T(2) * (xy * xy + xz * xz + yz * yz));
      }
    }
    cplx<float2> y[RR];
#pragma unroll
    for (int m = 0; m < RR; ++m) {
      const T ux = f[0][m], uy = f[1][m], uz = f[2][m];
      T o0, o1, o2, o3;
      if (c == 0) {
        const T wx = f[3][m], wy = f[4][m], wz = f[5][m];
        umax = fmaxf(umax, fmaxf(fabsf(ux), fmaxf(fabsf(uy), fabsf(uz))));
        o0 = uy * wz - uz * wy;   // (u x w)
        o1 = uz * wx - ux * wz;
        o2 = ux * wy - uy * wx;
        o3 = want_ke ? T(0.5) * (ux * ux + uy * uy + uz * uz) : T(0);
      } else if (c == 1) {
        o0 = nrm[m] * f[6][m]; o1 = nrm[m] * f[7][m]; o2 = nrm[m] * f[8][m]; o3 = nrm[m] * f[9][m];
      } else {
        o0 = nrm[m] * f[10][m];
        if (DEN) {
          const T rho = f[11][m];
          rmax = fmaxf(rmax, fabsf(rho));
          o1 = -rho * ux; o2 = -rho * uy; o3 = -rho * uz;
        } else {
          o1 = o2 = o3 = T(0);
        }
      }
      y[m] = mk(make_float2(o0, o2), make_float2(o1, o3));
    }
    dftR<RR, -1>(y);
#pragma unroll
    for (int m = 0; m < RR; ++m) P[c * PE + C::pix(i * RR + m, q)] = y[m];
  }
  if (I.adaptive) block_max_to_state<T, DEN>(I, umax, rmax, red);   // contains a __syncthreads
  else __syncthreads();

  // ---- forward pass 1 (radix R0, p = 8), in place: twiddles w^(ii m)
#pragma unroll 1
  for (int b = tid; b < 3 * LYZ * T0; b += NT) {
    const int ii = b % T0, ql = (b / T0) % LYZ, c = b / (T0 * LYZ);
    cplx<float2> x[R0];
#pragma unroll
    for (int m = 0; m < R0; ++m) x[m] = P[c * PE + C::pix(ii + T0 * m, ql)];
    if (ii != 0) {
#pragma unroll
      for (int m = 1; m < R0; ++m) {
        const cplx<T> w = I.twx[ii * m];
        x[m] = twmul2<-1>(x[m], make_float2(w.x, w.x), make_float2(w.y, w.y));
      }
    }
    dftR<R0, -1>(x);
#pragma unroll
    for (int m = 0; m < R0; ++m) P[c * PE + C::pix(ii + T0 * m, ql)] = x[m];
  }
  __syncthreads();

  // ---- unpack A = (Z_k + conj Z_{n-k})/2, B = -i (Z_k - conj Z_{n-k})/2 of both lines of
  // each pair; thread (q, i) writes k = i, i + TPL, ... of line q. Output 3 (kinetic
  // energy) only at stats/spectrum iterations.
  const long long row = (g0 + q) * KXP;
#pragma unroll 1
  for (int k = i; k < KXP; k += TPL) {
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      cplx<T> a0 = mk(T(0), T(0)), b0 = a0, a1 = a0, b1 = a0;
      if (k < Mx) {
        const cplx<float2> zk = P[c * PE + C::pix(k, q)];
        const cplx<float2> zm = P[c * PE + C::pix(k == 0 ? 0 : N - k, q)];
        // twice A and B: the forward z pass scales by 1/(2N)
        a0 = mk(zk.x.x + zm.x.x, zk.y.x - zm.y.x);
        b0 = mk(zk.y.x + zm.y.x, zm.x.x - zk.x.x);
        a1 = mk(zk.x.y + zm.x.y, zk.y.y - zm.y.y);
        b1 = mk(zk.y.y + zm.y.y, zm.x.y - zk.x.y);
      }
      const int o = 4 * c;
      I.wy[(long long)I.out_slot[o] * I.wys + row + k] = a0;
      if (o + 1 < NOUT) I.wy[(long long)I.out_slot[o + 1] * I.wys + row + k] = b0;
      if (o + 2 < NOUT) I.wy[(long long)I.out_slot[o + 2] * I.wys + row + k] = a1;
      if (o + 3 < NOUT && (o + 3 != 3 || want_ke)) I.wy[(long long)I.out_slot[o + 3] * I.wys + row + k] = b1;
    }
  }
}

template <int N, bool DEN>
__global__ void __launch_bounds__(XLes<N>::NT, XLesCfg<N>::MINB) k_x_les(Inst<float> I) {
  b_x_les<N, DEN>(I, Blk::here());
}

}  // namespace ffsgpu
