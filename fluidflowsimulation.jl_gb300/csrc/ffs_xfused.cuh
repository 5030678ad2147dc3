// Register-fused x pass for the velocity-only model in FP32 (realspace! +
// realspacecalculation! + find_max, models.jl:121-214, 228-280, utils.jl:247-258).
//
// The x transforms use a plan whose first and last radix agree, n = R * R2 * R
// (R2 = 1: two passes). Thread (q, i) of a CTA owns the elements j = i + m n/R, m < R,
// of (y,z) line q: they are the outputs of the last inverse radix pass and exactly the
// inputs of the first forward radix pass. So the last inverse pass, the products
// u x w (and 1/2 |u|^2 at stats iterations) and the first forward pass run in registers,
// with no shared-memory round trip between them:
//
//   global half spectra -> inverse pass 0 -> smem [-> middle pass -> smem]
//   -> registers: last inverse pass, products, forward pass 0 -> smem
//   [-> middle pass -> smem] -> last forward pass (in place) -> Hermitian unpack -> global
//
// Six real input fields ride as three complex lines (ux+i uy, uz+i wx, wy+i wz) and four
// outputs as two (Nx+i Ny, Nz+i ke). Shared lines are stored line-fastest with an odd
// line stride and a padding row every 16, which keeps the radix-R strided accesses of
// the register passes free of bank conflicts.
#pragma once
#include "ffs_kernels.cuh"

namespace ffsgpu {

__device__ __forceinline__ cplx<float> ldg_c(const cplx<float>* p) {
  const float2 v = __ldg(reinterpret_cast<const float2*>(p));
  return mk(v.x, v.y);
}

template <int N> struct XFusedCfg;
template <> struct XFusedCfg<128> { static constexpr int R = 8, R2 = 2, LYZ = 8, MINB = 4; };
template <> struct XFusedCfg<256> { static constexpr int R = 16, R2 = 1, LYZ = 8, MINB = 4; };
template <> struct XFusedCfg<512> { static constexpr int R = 8, R2 = 8, LYZ = 2, MINB = 3; };
template <> struct XFusedCfg<1024> { static constexpr int R = 8, R2 = 16, LYZ = 1, MINB = 3; };

template <int N> struct XFused {
  static constexpr int R = XFusedCfg<N>::R, R2 = XFusedCfg<N>::R2, LYZ = XFusedCfg<N>::LYZ;
  static constexpr int TPL = N / R;        // threads per (y,z) line
  static constexpr int NT = LYZ * TPL;     // threads per CTA
  static constexpr int NL = 3 * LYZ;       // complex lines per CTA
  static constexpr int LS = NL + 1;        // odd line stride
  static constexpr int NBUF = R2 > 1 ? 2 : 1;
  static size_t smem() { return sizeof(cplx<float>) * (size_t)NBUF * srows(N) * LS; }
};

// twiddle table of the register passes, [m][i] = exp(-2 pi i * i m / n), m < R, i < n/R
// (lanes i read consecutive entries)

template <int N>
__device__ __forceinline__ void b_x_fused(const Inst<float>& I, const Blk bk) {
  using T = float;
  using C = XFused<N>;
  constexpr int R = C::R, R2 = C::R2, LYZ = C::LYZ, TPL = C::TPL, NL = C::NL, LS = C::LS;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cplx<T>* s0 = reinterpret_cast<cplx<T>*>(smem_raw);
  cplx<T>* s1 = s0 + (R2 > 1 ? srows(N) * LS : 0);
  __shared__ T red[64];

  const int tid = threadIdx.x;
  const int q = tid / TPL, i = tid % TPL;
  const long long g = (long long)bk.x * LYZ + q;   // (y,z) line
  const int Mx = I.Mx, KXP = I.KXP;
  const long long it = I.st->iteration;
  const bool want_ke = ((it % I.dt_stat) == 0) || ((it % I.dt_spec) == 0);
  const cplx<T>* __restrict__ tw = I.twx;
  const cplx<T>* __restrict__ twr = I.twx_r;
  auto no_ld = [](int, int) -> cplx<T> { return mk(T(0), T(0)); };
  auto no_st = [](int, int, cplx<T>) {};

  // The CTA x_pf_dist ahead will most likely start when this one retires: bring its six
  // input slabs (LYZ consecutive lines each, contiguous) into L2 now, so that its pass-0
  // loads wait on L2 rather than DRAM.
  if (I.x_pf_dist > 0 && tid < 6) {
    const long long nb = (long long)bk.x + I.x_pf_dist;
    const long long ng = (long long)I.ny * I.nz / LYZ;
    if (nb < ng)
      prefetch_l2(I.wy + (long long)tid * I.wys + nb * LYZ * KXP, (unsigned)(sizeof(cplx<T>) * LYZ * KXP));
  }

  // ---- inverse pass 0 (radix R, no twiddles): Hermitian extension of the half spectra.
  // Read-only-path loads (each CTA reads its own lines before it writes any of them),
  // unrolled over the pairs so that the loads of the next pair are in flight during the
  // DFT of the current one.
#pragma unroll
  for (int p = 0; p < 3; ++p) {
    const cplx<T>* A = I.wy + (long long)(2 * p) * I.wys + g * KXP;
    const cplx<T>* B = I.wy + (long long)(2 * p + 1) * I.wys + g * KXP;
    cplx<T> x[R];
#pragma unroll
    for (int m = 0; m < R; ++m) {
      const int j = i + m * TPL;
      const bool cj = 2 * j > N;
      const int k = cj ? N - j : j;
      cplx<T> a = mk(T(0), T(0)), b = mk(T(0), T(0));
      if (k < Mx) { a = ldg_c(A + k); b = ldg_c(B + k); }
      if (k == 0 || 2 * k == N) { a.y = T(0); b.y = T(0); }   // c2r ignores Im at kx = 0 and n/2
      if (cj) { a.y = -a.y; b.y = -b.y; }
      x[m] = mk(a.x - b.y, a.y + b.x);
    }
    dftR<R, +1>(x);
    const int l = p * LYZ + q;
#pragma unroll
    for (int m = 0; m < R; ++m) s0[sidx(i * R + m, l, LS)] = x[m];
  }
  __syncthreads();
  if (R2 > 1) {   // middle radix pass, p = R
    fft_pass<R2, +1, NL, T>(N / R2, R, N / (R * R2), false, false, s0, s1, LS, tw, no_ld, no_st);
    __syncthreads();
  }
  cplx<T>* sl = R2 > 1 ? s1 : s0;   // buffer of the last radix pass

  // ---- last inverse pass in registers: fields (2p, 2p+1) at j = i + m TPL
  T f[6][R];
#pragma unroll
  for (int p = 0; p < 3; ++p) {
    const int l = p * LYZ + q;
    cplx<T> x[R];
#pragma unroll
    for (int m = 0; m < R; ++m) x[m] = sl[sidx(i + m * TPL, l, LS)];
#pragma unroll
    for (int m = 1; m < R; ++m) x[m] = x[m] * cjg(twr[m * TPL + i]);
    dftR<R, +1>(x);
#pragma unroll
    for (int m = 0; m < R; ++m) { f[2 * p][m] = x[m].x; f[2 * p + 1][m] = x[m].y; }
  }

  // ---- physical-space products (models.jl:224, 260) and max |u_i| (utils.jl:247-258)
  T umax = T(0);
#pragma unroll
  for (int m = 0; m < R; ++m) {
    const T ux = f[0][m], uy = f[1][m], uz = f[2][m], wx = f[3][m], wy = f[4][m], wz = f[5][m];
    umax = fmaxf(umax, fmaxf(fabsf(ux), fmaxf(fabsf(uy), fabsf(uz))));
    f[0][m] = uy * wz - uz * wy;
    f[1][m] = uz * wx - ux * wz;
    f[2][m] = ux * wy - uy * wx;
    f[3][m] = want_ke ? T(0.5) * (ux * ux + uy * uy + uz * uz) : T(0);
  }

  // ---- forward pass 0 in registers (radix R, no twiddles)
  cplx<T> y[2][R];
#pragma unroll
  for (int r = 0; r < 2; ++r) {
#pragma unroll
    for (int m = 0; m < R; ++m) y[r][m] = mk(f[2 * r][m], f[2 * r + 1][m]);
    dftR<R, -1>(y[r]);
  }
  cplx<T>* sf = s0;   // s0 is free when a middle pass exists; otherwise wait for all reads
  if (R2 == 1) __syncthreads();
#pragma unroll
  for (int r = 0; r < 2; ++r) {
    const int l = r * LYZ + q;
#pragma unroll
    for (int m = 0; m < R; ++m) sf[sidx(i * R + m, l, LS)] = y[r][m];
  }
  if (I.adaptive) block_max_to_state<T, false>(I, umax, T(0), red);   // contains a __syncthreads
  else __syncthreads();
  if (R2 > 1) {
    fft_pass<R2, -1, 2 * LYZ, T>(N / R2, R, N / (R * R2), false, false, s0, s1, LS, tw, no_ld, no_st);
    __syncthreads();
  }

  // ---- last forward pass (each thread rewrites the positions it read)
#pragma unroll 1
  for (int r = 0; r < 2; ++r) {
    const int l = r * LYZ + q;
    cplx<T> x[R];
#pragma unroll
    for (int m = 0; m < R; ++m) x[m] = sl[sidx(i + m * TPL, l, LS)];
#pragma unroll
    for (int m = 1; m < R; ++m) x[m] = x[m] * twr[m * TPL + i];
    dftR<R, -1>(x);
#pragma unroll
    for (int m = 0; m < R; ++m) sl[sidx(i + m * TPL, l, LS)] = x[m];
  }
  __syncthreads();

  // ---- unpack A = (Z_k + conj Z_{n-k})/2, B = -i (Z_k - conj Z_{n-k})/2 and store kx < KXP
  {
    const int wv = tid >> 5, lane = tid & 31;
    constexpr int NW = C::NT / 32;
#pragma unroll 1
    for (int l = wv; l < 2 * LYZ; l += NW) {   // l = r LYZ + q' carries outputs (2r, 2r+1)
      const int r = l / LYZ, qq = l % LYZ;
      const int oa = 2 * r, ob = 2 * r + 1;
      const bool wb = ob != 3 || want_ke;   // output 3 (kinetic energy) only at stats iterations
      const long long row = ((long long)bk.x * LYZ + qq) * KXP;
      cplx<T>* da = I.wy + (long long)I.out_slot[oa] * I.wys + row;
      cplx<T>* db = I.wy + (long long)I.out_slot[ob] * I.wys + row;
      for (int k = lane; k < KXP; k += 32) {
        cplx<T> a = mk(T(0), T(0)), b = mk(T(0), T(0));
        if (k < Mx) {
          const cplx<T> zk = sl[sidx(k, l, LS)];
          const cplx<T> zm = sl[sidx(k == 0 ? 0 : N - k, l, LS)];
          a = mk(T(0.5) * (zk.x + zm.x), T(0.5) * (zk.y - zm.y));
          b = mk(T(0.5) * (zk.y + zm.y), T(-0.5) * (zk.x - zm.x));
        }
        da[k] = a;
        if (wb) db[k] = b;
      }
    }
  }
}

template <int N>
__global__ void __launch_bounds__(XFused<N>::NT, XFusedCfg<N>::MINB) k_x_fused(Inst<float> I) {
  b_x_fused<N>(I, Blk::here());
}

}  // namespace ffsgpu
