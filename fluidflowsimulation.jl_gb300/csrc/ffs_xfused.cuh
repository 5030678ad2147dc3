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
// outputs as two (Nx+i Ny, Nz+i ke). The first two input lines and both output lines are
// transformed as pairs on the packed FP32 pipe (cplx<float2>: one instruction advances
// both lines); the third input line runs alone. Pairs live in shared memory as one
// 16-byte element per position (the "pair plane", XOR-swizzled so that the strided
// accesses of the register passes are free of bank conflicts), the third line in a plane
// of 8-byte elements with an odd line stride and a padding row every 16.
#pragma once
#include <type_traits>

#include "ffs_kernels.cuh"

namespace ffsgpu {

__device__ __forceinline__ cplx<float> ldg_c(const cplx<float>* p) {
  const float2 v = __ldg(reinterpret_cast<const float2*>(p));
  return mk(v.x, v.y);
}

// Hermitian extension of a half spectrum for the first inverse radix pass: thread i takes
// element j = i + m n/R (m < R) of the full line; it reads half-spectrum entry k and uses
// a + i b -> (a.x - s b.y, s a.y + b.x) for a line packing two real fields a, b, where
// s = 1 for j < n/2, -1 for j > n/2 (k = n - j, conjugate) and 0 where c2r ignores the
// imaginary part (k = 0, k = n/2). With m known at compile time only m = 0 and m = R/2
// need run-time tests.
template <int N, int R>
__device__ __forceinline__ void herm_index(int i, int m, int& k, float& s) {
  constexpr int TPL = N / R;
  const int j = i + m * TPL;
  if (m < R / 2) { k = j; s = (m == 0 && i == 0) ? 0.f : 1.f; }
  else if (m > R / 2) { k = N - j; s = -1.f; }
  else { k = N / 2 - i; s = i == 0 ? 0.f : -1.f; }
}

template <int N> struct XFusedCfg;
template <> struct XFusedCfg<64> { static constexpr int R = 8, R2 = 1, LYZ = 8, MINB = 8; };
template <> struct XFusedCfg<128> { static constexpr int R = 8, R2 = 2, LYZ = 8, MINB = 4; };
template <> struct XFusedCfg<256> { static constexpr int R = 16, R2 = 1, LYZ = 8, MINB = 4; };
template <> struct XFusedCfg<512> { static constexpr int R = 8, R2 = 8, LYZ = 2, MINB = 3; };
template <> struct XFusedCfg<1024> { static constexpr int R = 8, R2 = 16, LYZ = 1, MINB = 3; };

template <int N> struct XFused {
  static constexpr int R = XFusedCfg<N>::R, R2 = XFusedCfg<N>::R2, LYZ = XFusedCfg<N>::LYZ;
  static constexpr int LOG2R = R == 16 ? 4 : 3;
  static constexpr int TPL = N / R;        // threads per (y,z) line
  static constexpr int NT = LYZ * TPL;     // threads per CTA
  static constexpr int NBUF = R2 > 1 ? 2 : 1;
  static constexpr int PE = N * LYZ;                   // 16-byte elements of one pair plane
  static constexpr int QLS = LYZ == 1 ? 1 : LYZ + 1;   // odd line stride of a single plane
  static constexpr int QE = (N + (N >> 4) + 1) * QLS;  // 8-byte elements of one single plane
  static size_t smem() { return (size_t)NBUF * (16 * (size_t)PE + 8 * (size_t)QE); }

  // Pair-plane position of element j of line q. Rows of 128 bytes (8 elements: the LYZ
  // lines of 1, 2 or 4 consecutive j) with the column XOR-ed by a function of the row, so
  // that each quarter warp (the unit of a 16-byte shared access) touches 8 distinct bank
  // groups both for 8 consecutive j (register passes, middle passes, unpack) and for j
  // stepping by R (the stores of pass 0).
  static __device__ __forceinline__ int pix(int j, int q) {
    if constexpr (LYZ == 8) {
      return j * 8 + (q ^ ((j ^ (j >> LOG2R)) & 7));
    } else if constexpr (LYZ == 2) {
      const int s = j >> 2, w = ((j & 3) << 1) | q;
      return s * 8 + (w ^ (((s >> 1) ^ (s & 1)) & 7));
    } else {
      const int s = j >> 3;
      return s * 8 + ((j & 7) ^ (s & 7));
    }
  }
};

// One Stockham middle pass (radix R2, sub-transform length p = R entering, T_ = n/R2
// butterflies per line) over the LYZ lines of a pair plane or, with PAIR false, of a
// single plane. tw: exp(-2 pi i t / n).
template <int N, bool PAIR, int DIR>
__device__ __forceinline__ void xf_mid_pass(const void* in_, void* out_, const cplx<float>* __restrict__ tw) {
  using C = XFused<N>;
  constexpr int R = C::R, R2 = C::R2, LYZ = C::LYZ, T_ = N / R2, p = R, tws = N / (R * R2);
  using V = typename std::conditional<PAIR, cplx<float2>, cplx<float>>::type;
  const V* in = reinterpret_cast<const V*>(in_);
  V* out = reinterpret_cast<V*>(out_);
  auto at = [](int j, int l) { return PAIR ? C::pix(j, l) : sidx(j, l, C::QLS); };
#pragma unroll 1
  for (int b = threadIdx.x; b < LYZ * T_; b += C::NT) {
    const int l = b % LYZ, i = b / LYZ;
    const int k = i & (p - 1);
    V x[R2];
#pragma unroll
    for (int m = 0; m < R2; ++m) x[m] = in[at(i + m * T_, l)];
    if (k != 0) {
#pragma unroll
      for (int m = 1; m < R2; ++m) {
        const cplx<float> w = tw[k * m * tws];
        if constexpr (PAIR) x[m] = twmul2<DIR>(x[m], make_float2(w.x, w.x), make_float2(w.y, w.y));
        else x[m] = twmul1<DIR>(x[m], w.x, w.y);
      }
    }
    dftR<R2, DIR>(x);
    const int j = (i - k) * R2 + k;
#pragma unroll
    for (int m = 0; m < R2; ++m) out[at(j + m * p, l)] = x[m];
  }
}

// Register-pass twiddles, [m][i] = (c, c, s, s) with exp(-2 pi i * i m / n) = (c, s),
// m < R, i < n/R (lanes i read consecutive entries)

template <int N>
__device__ __forceinline__ void b_x_fused(const Inst<float>& I, const Blk bk) {
  using T = float;
  using C = XFused<N>;
  constexpr int R = C::R, R2 = C::R2, LYZ = C::LYZ, TPL = C::TPL, QLS = C::QLS;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  // [pair plane 0][pair plane 1][single plane 0][single plane 1] (second of each when R2 > 1)
  cplx<float2>* P0 = reinterpret_cast<cplx<float2>*>(smem_raw);
  cplx<float2>* P1 = P0 + (R2 > 1 ? C::PE : 0);
  cplx<T>* Q0 = reinterpret_cast<cplx<T>*>(P0 + C::NBUF * C::PE);
  cplx<T>* Q1 = Q0 + (R2 > 1 ? C::QE : 0);
  cplx<float2>* Pl = R2 > 1 ? P1 : P0;   // planes the last radix passes read
  cplx<T>* Ql = R2 > 1 ? Q1 : Q0;
  __shared__ T red[64];

  const int tid = threadIdx.x;
  const int q = tid / TPL, i = tid % TPL;
  const long long g = (long long)bk.x * LYZ + q;   // (y,z) line
  const int Mx = I.Mx, KXP = I.KXP;
  const long long it = I.st->iteration;
  const bool want_ke = ((it % I.dt_stat) == 0) || ((it % I.dt_spec) == 0);
  const cplx<float2>* __restrict__ twr = reinterpret_cast<const cplx<float2>*>(I.twx_r);

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
  // Read-only-path loads (each CTA reads its own lines before it writes any of them).
  {
    const cplx<T>* F0 = I.wy + g * KXP;
    const long long fs = I.wys;
    cplx<float2> x[R];
#pragma unroll
    for (int m = 0; m < R; ++m) {
      int k;
      T sg;
      herm_index<N, R>(i, m, k, sg);
      cplx<T> a0 = mk(T(0), T(0)), b0 = a0, a1 = a0, b1 = a0;
      if (k < Mx) { a0 = ldg_c(F0 + k); b0 = ldg_c(F0 + fs + k); a1 = ldg_c(F0 + 2 * fs + k); b1 = ldg_c(F0 + 3 * fs + k); }
      x[m] = mk(make_float2(fmaf(-sg, b0.y, a0.x), fmaf(-sg, b1.y, a1.x)),
                make_float2(fmaf(sg, a0.y, b0.x), fmaf(sg, a1.y, b1.x)));
    }
    dftR<R, +1>(x);
#pragma unroll
    for (int m = 0; m < R; ++m) P0[C::pix(i * R + m, q)] = x[m];
  }
  {
    const cplx<T>* A = I.wy + 4 * I.wys + g * KXP;
    const cplx<T>* B = A + I.wys;
    cplx<T> x[R];
#pragma unroll
    for (int m = 0; m < R; ++m) {
      int k;
      T sg;
      herm_index<N, R>(i, m, k, sg);
      cplx<T> a = mk(T(0), T(0)), b = a;
      if (k < Mx) { a = ldg_c(A + k); b = ldg_c(B + k); }
      x[m] = mk(fmaf(-sg, b.y, a.x), fmaf(sg, a.y, b.x));
    }
    dftR<R, +1>(x);
#pragma unroll
    for (int m = 0; m < R; ++m) Q0[sidx(i * R + m, q, QLS)] = x[m];
  }
  __syncthreads();
  if constexpr (R2 > 1) {
    xf_mid_pass<N, true, +1>(P0, P1, I.twx);
    xf_mid_pass<N, false, +1>(Q0, Q1, I.twx);
    __syncthreads();
  }

  // ---- last inverse pass in registers: fields 0..5 at j = i + m TPL
  T f[6][R];
  {
    cplx<float2> x[R];
#pragma unroll
    for (int m = 0; m < R; ++m) x[m] = Pl[C::pix(i + m * TPL, q)];
#pragma unroll
    for (int m = 1; m < R; ++m) { const cplx<float2> w = twr[m * TPL + i]; x[m] = twmul2<+1>(x[m], w.x, w.y); }
    dftR<R, +1>(x);
#pragma unroll
    for (int m = 0; m < R; ++m) { f[0][m] = x[m].x.x; f[1][m] = x[m].y.x; f[2][m] = x[m].x.y; f[3][m] = x[m].y.y; }
  }
  {
    cplx<T> x[R];
#pragma unroll
    for (int m = 0; m < R; ++m) x[m] = Ql[sidx(i + m * TPL, q, QLS)];
#pragma unroll
    for (int m = 1; m < R; ++m) { const cplx<float2> w = twr[m * TPL + i]; x[m] = twmul1<+1>(x[m], w.x.x, w.y.x); }
    dftR<R, +1>(x);
#pragma unroll
    for (int m = 0; m < R; ++m) { f[4][m] = x[m].x; f[5][m] = x[m].y; }
  }

  // ---- physical-space products (models.jl:224, 260) and max |u_i| (utils.jl:247-258),
  // packed as the forward pair (Nx + i Ny, Nz + i ke)
  T umax = T(0);
  cplx<float2> y[R];
#pragma unroll
  for (int m = 0; m < R; ++m) {
    const T ux = f[0][m], uy = f[1][m], uz = f[2][m], wx = f[3][m], wy = f[4][m], wz = f[5][m];
    umax = fmaxf(umax, fmaxf(fabsf(ux), fmaxf(fabsf(uy), fabsf(uz))));
    const T nx = uy * wz - uz * wy, ny = uz * wx - ux * wz, nz = ux * wy - uy * wx;
    const T ke = want_ke ? T(0.5) * (ux * ux + uy * uy + uz * uz) : T(0);
    y[m] = mk(make_float2(nx, nz), make_float2(ny, ke));
  }

  // ---- forward pass 0 in registers (radix R, no twiddles)
  dftR<R, -1>(y);
  if (R2 == 1) __syncthreads();   // P0 is the plane the register pass just read
#pragma unroll
  for (int m = 0; m < R; ++m) P0[C::pix(i * R + m, q)] = y[m];
  if (I.adaptive) block_max_to_state<T, false>(I, umax, T(0), red);   // contains a __syncthreads
  else __syncthreads();
  if constexpr (R2 > 1) {
    xf_mid_pass<N, true, -1>(P0, P1, I.twx);
    __syncthreads();
  }

  // ---- last forward pass (each thread rewrites the positions it read)
  {
    cplx<float2> x[R];
#pragma unroll
    for (int m = 0; m < R; ++m) x[m] = Pl[C::pix(i + m * TPL, q)];
#pragma unroll
    for (int m = 1; m < R; ++m) { const cplx<float2> w = twr[m * TPL + i]; x[m] = twmul2<-1>(x[m], w.x, w.y); }
    dftR<R, -1>(x);
#pragma unroll
    for (int m = 0; m < R; ++m) Pl[C::pix(i + m * TPL, q)] = x[m];
  }
  __syncthreads();

  // ---- unpack A = (Z_k + conj Z_{n-k})/2, B = -i (Z_k - conj Z_{n-k})/2 of both lines of
  // the pair and store kx < KXP; thread (q, i) writes k = i, i + TPL, ... of line q
  {
    const long long row = g * KXP;
    cplx<T>* d0 = I.wy + (long long)I.out_slot[0] * I.wys + row;
    cplx<T>* d1 = I.wy + (long long)I.out_slot[1] * I.wys + row;
    cplx<T>* d2 = I.wy + (long long)I.out_slot[2] * I.wys + row;
    cplx<T>* d3 = I.wy + (long long)I.out_slot[3] * I.wys + row;
#pragma unroll 1
    for (int k = i; k < KXP; k += TPL) {
      cplx<T> a0 = mk(T(0), T(0)), b0 = a0, a1 = a0, b1 = a0;
      if (k < Mx) {
        const cplx<float2> zk = Pl[C::pix(k, q)];
        const cplx<float2> zm = Pl[C::pix(k == 0 ? 0 : N - k, q)];
        // twice A and B: the forward z pass scales by 1/(2N)
        a0 = mk(zk.x.x + zm.x.x, zk.y.x - zm.y.x);
        b0 = mk(zk.y.x + zm.y.x, zm.x.x - zk.x.x);
        a1 = mk(zk.x.y + zm.x.y, zk.y.y - zm.y.y);
        b1 = mk(zk.y.y + zm.y.y, zm.x.y - zk.x.y);
      }
      d0[k] = a0;
      d1[k] = b0;
      d2[k] = a1;
      if (want_ke) d3[k] = b1;   // output 3 (kinetic energy) only at stats iterations
    }
  }
}

template <int N>
__global__ void __launch_bounds__(XFused<N>::NT, XFusedCfg<N>::MINB) k_x_fused(Inst<float> I) {
  b_x_fused<N>(I, Blk::here());
}

}  // namespace ffsgpu
