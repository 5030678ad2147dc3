// Shared-memory Stockham FFT core for line batches (sm_103a).
//
// A CTA transforms L lines of length n.  Line l, element j lives in shared memory at
// buf[sidx(j, l, LS)] (lines fastest, one padding row every 16), so a warp touches
// consecutive addresses.
// Pass 0 reads its inputs through a loader functor (straight from global memory, with
// any spectral prologue fused in) and the last pass hands its outputs to a storer
// functor (global store, pruning, or epilogue math), so a two-pass transform
// (n = R0 * R1) makes a single round trip through shared memory.
//
// Formulation (radix R, sub-transform length p, T = n / R butterflies per line):
//   k = i mod p;  x_m = in[i + m T] * w^(k m n/(p R));  X = DFT_R(x);
//   out[(i - k) R + k + m p] = X_m
// with w = exp(-2 pi i / n) for the forward transform and its conjugate for the
// inverse.  Output comes out in natural order after the last pass.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace ffsgpu {

// aligned to its size, so that one complex moves in one 8-byte (float) or 16-byte (double)
// load or store instead of two
template <typename T> struct alignas(2 * sizeof(T)) cplx { T x, y; };

template <typename T> __device__ __forceinline__ cplx<T> mk(T a, T b) { cplx<T> r; r.x = a; r.y = b; return r; }
template <typename T> __device__ __forceinline__ cplx<T> operator+(cplx<T> a, cplx<T> b) { return mk(a.x + b.x, a.y + b.y); }
template <typename T> __device__ __forceinline__ cplx<T> operator-(cplx<T> a, cplx<T> b) { return mk(a.x - b.x, a.y - b.y); }
template <typename T> __device__ __forceinline__ cplx<T> operator*(cplx<T> a, cplx<T> b) {
  return mk(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
template <typename T> __device__ __forceinline__ cplx<T> scl(cplx<T> a, T s) { return mk(a.x * s, a.y * s); }

// Packed FP32 (sm_100 and later): a float2 is two independent lanes, and cplx<float2>
// carries two complex numbers (re of both, im of both), so the same DFT code advances two
// lines with half the FP32 instructions. Each lane rounds exactly as the scalar operation.
__device__ __forceinline__ float2 operator+(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 operator-(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }
__device__ __forceinline__ float2 operator*(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 operator-(float2 a) { return __fmul2_rn(a, make_float2(-1.f, -1.f)); }

// a constant in the arithmetic type (both lanes for float2)
template <typename T> __device__ __forceinline__ T cst(double v) { return T(v); }
template <> __device__ __forceinline__ float2 cst<float2>(double v) { return make_float2((float)v, (float)v); }

// a * b + c, rounded once
__device__ __forceinline__ float fma_(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double fma_(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float2 fma_(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
template <typename T> __device__ __forceinline__ cplx<T> cjg(cplx<T> a) { return mk(a.x, -a.y); }
// multiply by +i (DIR=+1) or -i (DIR=-1)
template <int DIR, typename T> __device__ __forceinline__ cplx<T> mul_i(cplx<T> a) {
  return DIR > 0 ? mk(-a.y, a.x) : mk(a.y, -a.x);
}

struct FftPlan {
  int n;      // transform length
  int np;     // number of passes
  int r[4];   // radices, product == n
  int tpl;    // threads per line = n / largest radix
  int T[4];   // butterflies per line in each pass, n / r
  int p[4];   // sub-transform length entering each pass (a power of two: radix 3 comes last)
  int tws[4]; // twiddle table stride, n / (p r)
};

// Shared-memory position of element j of line l: one padding row every 16 rows keeps
// the stride-R writes of the first pass free of bank conflicts. Buffers hold
// srows(n) * LS elements.
__host__ __device__ __forceinline__ int sidx(int j, int l, int LS) { return (j + (j >> 4)) * LS + l; }
__host__ __device__ __forceinline__ int srows(int n) { return n + (n >> 4) + 1; }

// Division by a runtime constant with a multiply-high (for 0 <= x < 2^31).
struct FastDiv {
  unsigned d, m, s;
};
__host__ inline FastDiv make_fastdiv(unsigned d) {
  FastDiv f;
  f.d = d;
  unsigned s = 0;
  while ((1ull << s) < d) ++s;
  f.s = s;
  f.m = (unsigned)(((1ull << 32) * ((1ull << s) - d)) / d + 1);
  return f;
}
__device__ __forceinline__ unsigned fdiv(unsigned x, const FastDiv& f) {
  return (__umulhi(x, f.m) + x) >> f.s;
}

// ---------------------------------------------------------------------------------
// Small DFTs in registers. DIR = -1 forward (exp(-i..)), +1 inverse.
// Constants are exact mathematical values (cos/sin of multiples of pi/8, sqrt(3)/2).
// ---------------------------------------------------------------------------------
#define FFS_C8 0.92387953251128675612818318939678829   /* cos(pi/8) */
#define FFS_S8 0.38268343236508977172845998403039887   /* sin(pi/8) */
#define FFS_R2 0.70710678118654752440084436210484904   /* sqrt(1/2) */
#define FFS_R3 0.86602540378443864676372317075293618   /* sqrt(3)/2 */

template <int DIR, typename T> __device__ __forceinline__ void dft2(cplx<T>& a, cplx<T>& b) {
  cplx<T> t = a; a = t + b; b = t - b;
}

template <int DIR, typename T> __device__ __forceinline__ void dft4(cplx<T>& x0, cplx<T>& x1, cplx<T>& x2, cplx<T>& x3) {
  cplx<T> a0 = x0 + x2, a1 = x0 - x2, a2 = x1 + x3, d = x1 - x3;
  x0 = a0 + a2; x2 = a0 - a2;
  // x1 = a1 + (DIR i) d, x3 = a1 - (DIR i) d, with the rotation folded into the adds
  if (DIR > 0) { x1 = mk(a1.x - d.y, a1.y + d.x); x3 = mk(a1.x + d.y, a1.y - d.x); }
  else { x1 = mk(a1.x + d.y, a1.y - d.x); x3 = mk(a1.x - d.y, a1.y + d.x); }
}

template <int DIR, typename T> __device__ __forceinline__ void dft3(cplx<T>& x0, cplx<T>& x1, cplx<T>& x2) {
  const T nh = cst<T>(-0.5), s = cst<T>(FFS_R3), ns = cst<T>(-FFS_R3);
  cplx<T> t1 = x1 + x2, t2 = x1 - x2;
  cplx<T> c = mk(fma_(nh, t1.x, x0.x), fma_(nh, t1.y, x0.y));
  // d = (DIR i) sqrt(3)/2 t2
  cplx<T> d = DIR > 0 ? mk(t2.y * ns, t2.x * s) : mk(t2.y * s, t2.x * ns);
  x0 = x0 + t1; x1 = c + d; x2 = c - d;
}

// multiply by exp(DIR * 2 pi i t / 8), t = 1,2,3
template <int DIR, int t, typename T> __device__ __forceinline__ cplx<T> w8(cplx<T> a) {
  const T r = cst<T>(FFS_R2), nr = cst<T>(-FFS_R2);
  if (t == 1) return DIR > 0 ? mk(r * (a.x - a.y), r * (a.x + a.y)) : mk(r * (a.x + a.y), r * (a.y - a.x));
  if (t == 2) return mul_i<DIR>(a);
  // t == 3: exp(DIR 3 pi i/4) = (-r, DIR r)
  return DIR > 0 ? mk(nr * (a.x + a.y), r * (a.x - a.y)) : mk(r * (a.y - a.x), nr * (a.x + a.y));
}

template <int DIR, typename T> __device__ __forceinline__ void dft8(cplx<T>* x) {
  dft4<DIR>(x[0], x[2], x[4], x[6]);
  dft4<DIR>(x[1], x[3], x[5], x[7]);
  cplx<T> o1 = w8<DIR, 1>(x[3]), o2 = w8<DIR, 2>(x[5]), o3 = w8<DIR, 3>(x[7]);
  cplx<T> e0 = x[0], e1 = x[2], e2 = x[4], e3 = x[6], o0 = x[1];
  x[0] = e0 + o0; x[4] = e0 - o0;
  x[1] = e1 + o1; x[5] = e1 - o1;
  x[2] = e2 + o2; x[6] = e2 - o2;
  x[3] = e3 + o3; x[7] = e3 - o3;
}

// multiply by exp(DIR * 2 pi i t / 16) for t in {1,2,3,4,6,9}
template <int DIR, int t, typename T> __device__ __forceinline__ cplx<T> w16(cplx<T> a) {
  if constexpr (t == 0) return a;
  else if constexpr (t == 2) return w8<DIR, 1>(a);
  else if constexpr (t == 4) return mul_i<DIR>(a);
  else if constexpr (t == 6) return w8<DIR, 3>(a);
  else {
    // general: (cos th, DIR sin th) * a; t == 9: cos(9pi/8) = -cos(pi/8), sin(9pi/8) = -sin(pi/8)
    constexpr double cr = t == 1 ? FFS_C8 : t == 3 ? FFS_S8 : -FFS_C8;
    constexpr double s0 = t == 1 ? FFS_S8 : t == 3 ? FFS_C8 : -FFS_S8;
    constexpr double si = DIR > 0 ? s0 : -s0;
    return mk(fma_(a.x, cst<T>(cr), a.y * cst<T>(-si)), fma_(a.x, cst<T>(si), a.y * cst<T>(cr)));
  }
}

template <int DIR, typename T> __device__ __forceinline__ void dft16(cplx<T>* x) {
  // x index m = 4 m1 + m2, output k = k1 + 4 k2
  dft4<DIR>(x[0], x[4], x[8], x[12]);
  dft4<DIR>(x[1], x[5], x[9], x[13]);
  dft4<DIR>(x[2], x[6], x[10], x[14]);
  dft4<DIR>(x[3], x[7], x[11], x[15]);
  // now x[4 k1 + m2] holds Y[m2][k1]; twiddle by W16^(m2 k1)
  x[5] = w16<DIR, 1>(x[5]); x[9] = w16<DIR, 2>(x[9]); x[13] = w16<DIR, 3>(x[13]);
  x[6] = w16<DIR, 2>(x[6]); x[10] = w16<DIR, 4>(x[10]); x[14] = w16<DIR, 6>(x[14]);
  x[7] = w16<DIR, 3>(x[7]); x[11] = w16<DIR, 6>(x[11]); x[15] = w16<DIR, 9>(x[15]);
  // Y[m2][k1] at x[m2 + 4 k1]; DFT4 over m2 for each k1
  dft4<DIR>(x[0], x[1], x[2], x[3]);
  dft4<DIR>(x[4], x[5], x[6], x[7]);
  dft4<DIR>(x[8], x[9], x[10], x[11]);
  dft4<DIR>(x[12], x[13], x[14], x[15]);
  // result X[k1 + 4 k2] sits at x[4 k1 + k2]: transpose the 4x4
  cplx<T> t;
#define FFS_SW(a, b) t = x[a]; x[a] = x[b]; x[b] = t;
  FFS_SW(1, 4) FFS_SW(2, 8) FFS_SW(3, 12) FFS_SW(6, 9) FFS_SW(7, 13) FFS_SW(11, 14)
#undef FFS_SW
}

template <int R, int DIR, typename T> __device__ __forceinline__ void dftR(cplx<T>* x) {
  if constexpr (R == 2) dft2<DIR>(x[0], x[1]);
  else if constexpr (R == 3) dft3<DIR>(x[0], x[1], x[2]);
  else if constexpr (R == 4) dft4<DIR>(x[0], x[1], x[2], x[3]);
  else if constexpr (R == 8) dft8<DIR>(x);
  else if constexpr (R == 16) dft16<DIR>(x);
}

// ---------------------------------------------------------------------------------
// One Stockham pass over L lines.
//   first: inputs come from the loader ld(l, j) instead of shared memory.
//   last:  outputs go to the storer st(l, j, v) instead of shared memory.
// In the last pass p * R = n, so every butterfly writes exactly the positions it read
// (j = i); a storer may therefore write back into the buffer the last pass reads.
// tw: table exp(-2 pi i t / n), t in [0, n).
// ---------------------------------------------------------------------------------
// NT > 0: the CTA has exactly NT threads (compile-time loop bounds).
template <int R, int DIR, int L, typename T, class LD, class ST, int NT = 0>
__device__ __forceinline__ void fft_pass(int T_, int p, int tws, bool first, bool last, const cplx<T>* in,
                                         cplx<T>* out, int LS, const cplx<T>* __restrict__ tw, LD& ld, ST& st) {
  const int nb = L * T_;
  const int stride = NT > 0 ? NT : (int)blockDim.x;
  for (int b = threadIdx.x; b < nb; b += stride) {
    const int l = b % L, i = b / L;
    const int k = i & (p - 1);
    cplx<T> x[R];
    if (first) {
#pragma unroll
      for (int m = 0; m < R; ++m) x[m] = ld(l, i + m * T_);
    } else {
#pragma unroll
      for (int m = 0; m < R; ++m) x[m] = in[sidx(i + m * T_, l, LS)];
      if (k != 0) {
#pragma unroll
        for (int m = 1; m < R; ++m) {
          cplx<T> w = tw[k * m * tws];
          if (DIR > 0) w.y = -w.y;
          x[m] = x[m] * w;
        }
      }
    }
    dftR<R, DIR>(x);
    const int j = (i - k) * R + k;
    if (last) {
#pragma unroll
      for (int m = 0; m < R; ++m) st(l, j + m * p, x[m]);
    } else {
#pragma unroll
      for (int m = 0; m < R; ++m) out[sidx(j + m * p, l, LS)] = x[m];
    }
  }
}

// The shared buffer the last pass reads (and an in-place storer may write): s0 for one-
// and two-pass plans, alternating s0/s1 for longer plans.
template <typename T> __device__ __forceinline__ cplx<T>* fft_result_buffer(const FftPlan& P, cplx<T>* s0, cplx<T>* s1) {
  return P.np >= 2 && ((P.np - 2) & 1) ? s1 : s0;
}

// Runs the whole plan. Pass 0 writes s0, later passes alternate s0/s1 (s1 is touched
// only for plans of three or more passes); both hold srows(n) * LS elements laid out by
// sidx(). Ends with a __syncthreads().
template <int DIR, int L, typename T, class LD, class ST>
__device__ void fft_lines(const FftPlan& P, cplx<T>* s0, cplx<T>* s1, int LS, const cplx<T>* __restrict__ tw, LD ld,
                          ST st) {
  for (int pass = 0; pass < P.np; ++pass) {
    const bool first = pass == 0, last = pass == P.np - 1;
    const cplx<T>* in = ((pass - 1) & 1) ? s1 : s0;
    cplx<T>* out = (pass & 1) ? s1 : s0;
    const int T_ = P.T[pass], p = P.p[pass], tws = P.tws[pass];
    switch (P.r[pass]) {
      case 16: fft_pass<16, DIR, L, T>(T_, p, tws, first, last, in, out, LS, tw, ld, st); break;
      case 8: fft_pass<8, DIR, L, T>(T_, p, tws, first, last, in, out, LS, tw, ld, st); break;
      case 4: fft_pass<4, DIR, L, T>(T_, p, tws, first, last, in, out, LS, tw, ld, st); break;
      case 3: fft_pass<3, DIR, L, T>(T_, p, tws, first, last, in, out, LS, tw, ld, st); break;
      default: fft_pass<2, DIR, L, T>(T_, p, tws, first, last, in, out, LS, tw, ld, st); break;
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------------
// Compile-time plans for the common power-of-two lengths (the radices make_plan picks):
// every pass constant folds, and the CTA size is the plan's threads per line x L.
// ---------------------------------------------------------------------------------
template <int N> struct CtPlan { static constexpr int np = 0; };
template <> struct CtPlan<32> { static constexpr int np = 2, r0 = 8, r1 = 4, r2 = 0, rmax = 8; };
template <> struct CtPlan<48> { static constexpr int np = 3, r0 = 4, r1 = 4, r2 = 3, rmax = 4; };
template <> struct CtPlan<64> { static constexpr int np = 2, r0 = 8, r1 = 8, r2 = 0, rmax = 8; };
template <> struct CtPlan<96> { static constexpr int np = 3, r0 = 8, r1 = 4, r2 = 3, rmax = 8; };
template <> struct CtPlan<128> { static constexpr int np = 2, r0 = 16, r1 = 8, r2 = 0, rmax = 16; };
template <> struct CtPlan<256> { static constexpr int np = 2, r0 = 16, r1 = 16, r2 = 0, rmax = 16; };
template <> struct CtPlan<512> { static constexpr int np = 3, r0 = 8, r1 = 8, r2 = 8, rmax = 8; };
template <> struct CtPlan<1024> { static constexpr int np = 3, r0 = 16, r1 = 8, r2 = 8, rmax = 16; };

template <int N> constexpr bool ct_plan_ok() { return CtPlan<N>::np > 0; }
template <int N> constexpr int ct_tpl() { return N / CtPlan<N>::rmax; }

// LS: line stride in shared memory; NTB: threads of the CTA (0: L * ct_tpl<N>()).
template <int DIR, int L, typename T, int N, class LD, class ST, int LS = L, int NTB = 0>
__device__ __forceinline__ void fft_lines_ct(cplx<T>* s0, cplx<T>* s1, const cplx<T>* __restrict__ tw, LD ld, ST st) {
  using C = CtPlan<N>;
  constexpr int NT = NTB > 0 ? NTB : L * ct_tpl<N>();
  constexpr int R0 = C::r0, R1 = C::r1, R2 = C::r2;
  // pass 0: p = 1
  fft_pass<R0, DIR, L, T, LD, ST, NT>(N / R0, 1, N / R0, true, false, s0, s0, LS, tw, ld, st);
  __syncthreads();
  if constexpr (C::np == 2) {
    fft_pass<R1, DIR, L, T, LD, ST, NT>(N / R1, R0, 1, false, true, s0, s1, LS, tw, ld, st);
    __syncthreads();
  } else {
    fft_pass<R1, DIR, L, T, LD, ST, NT>(N / R1, R0, N / (R0 * R1), false, false, s0, s1, LS, tw, ld, st);
    __syncthreads();
    fft_pass<R2, DIR, L, T, LD, ST, NT>(N / R2, R0 * R1, 1, false, true, s1, s0, LS, tw, ld, st);
    __syncthreads();
  }
}

// v * w (DIR < 0) or v * conj(w) (DIR > 0) for both lanes of v, with w = (c, s) given as
// C = (c, c), S = (s, s)
template <int DIR>
__device__ __forceinline__ cplx<float2> twmul2(cplx<float2> v, float2 C, float2 S) {
  const float2 NS = -S;
  const float2 P = v.x * C, Q = v.y * C;
  if (DIR < 0) return mk(fma_(v.y, NS, P), fma_(v.x, S, Q));
  return mk(fma_(v.y, S, P), fma_(v.x, NS, Q));
}
template <int DIR>
__device__ __forceinline__ cplx<float> twmul1(cplx<float> v, float c, float s) {
  if (DIR < 0) return mk(fmaf(v.y, -s, v.x * c), fmaf(v.x, s, v.y * c));
  return mk(fmaf(v.y, s, v.x * c), fmaf(v.x, -s, v.y * c));
}

// ---------------------------------------------------------------------------------
// Paired lines (FP32, compile-time plans): the L = 2 LP lines of a CTA as LP pairs
// (2 lp, 2 lp + 1), each pair transformed at once on the packed FP32 pipe by LP * tpl
// threads. Shared memory holds one 16-byte cplx<float2> per (position, pair); row j (LP
// elements) sits at row j ^ ((j >> S) & 1), S = log2 of the first radix, so that the two
// rows a quarter warp touches in every pass (j and j + 1, or j and j + R0 in the first
// pass) fall in opposite halves of the banks. The loader ld2(lp, j) returns and the
// storer st2(lp, j, v) takes both lines of a pair.
// ---------------------------------------------------------------------------------
template <int N> constexpr int ct_log2r0() {
  return CtPlan<N>::r0 == 16 ? 4 : CtPlan<N>::r0 == 8 ? 3 : CtPlan<N>::r0 == 4 ? 2 : 1;
}
template <int N, int LP> __device__ __forceinline__ int ppos(int j, int lp) {
  return (j ^ ((j >> ct_log2r0<N>()) & 1)) * LP + lp;
}

template <int R, int DIR, int LP, int N, class LD, class ST, int NT>
__device__ __forceinline__ void fft_pass2(int T_, int p, int tws, bool first, bool last, const cplx<float2>* in,
                                          cplx<float2>* out, const cplx<float>* __restrict__ tw, LD& ld, ST& st) {
#pragma unroll 1
  for (int b = threadIdx.x; b < LP * T_; b += NT) {
    const int lp = b % LP, i = b / LP;
    const int k = i & (p - 1);
    cplx<float2> x[R];
    if (first) {
#pragma unroll
      for (int m = 0; m < R; ++m) x[m] = ld(lp, i + m * T_);
    } else {
#pragma unroll
      for (int m = 0; m < R; ++m) x[m] = in[ppos<N, LP>(i + m * T_, lp)];
      if (k != 0) {
#pragma unroll
        for (int m = 1; m < R; ++m) {
          const cplx<float> w = tw[k * m * tws];
          x[m] = twmul2<DIR>(x[m], make_float2(w.x, w.x), make_float2(w.y, w.y));
        }
      }
    }
    dftR<R, DIR>(x);
    const int j = (i - k) * R + k;
    if (last) {
#pragma unroll
      for (int m = 0; m < R; ++m) st(lp, j + m * p, x[m]);
    } else {
#pragma unroll
      for (int m = 0; m < R; ++m) out[ppos<N, LP>(j + m * p, lp)] = x[m];
    }
  }
}

// Whole compile-time plan over LP pairs; s0 (and s1 for three-pass plans) hold N * LP
// elements. Ends with a __syncthreads().
template <int DIR, int LP, int N, class LD, class ST>
__device__ __forceinline__ void fft_lines_ct2(cplx<float2>* s0, cplx<float2>* s1, const cplx<float>* __restrict__ tw,
                                              LD ld, ST st) {
  using C = CtPlan<N>;
  constexpr int NT = LP * ct_tpl<N>();
  constexpr int R0 = C::r0, R1 = C::r1, R2 = C::r2;
  fft_pass2<R0, DIR, LP, N, LD, ST, NT>(N / R0, 1, N / R0, true, false, s0, s0, tw, ld, st);
  __syncthreads();
  if constexpr (C::np == 2) {
    fft_pass2<R1, DIR, LP, N, LD, ST, NT>(N / R1, R0, 1, false, true, s0, s1, tw, ld, st);
    __syncthreads();
  } else {
    fft_pass2<R1, DIR, LP, N, LD, ST, NT>(N / R1, R0, N / (R0 * R1), false, false, s0, s1, tw, ld, st);
    __syncthreads();
    fft_pass2<R2, DIR, LP, N, LD, ST, NT>(N / R2, R0 * R1, 1, false, true, s1, s0, tw, ld, st);
    __syncthreads();
  }
}

// 16-byte global accesses of a line pair (two adjacent complex values)
__device__ __forceinline__ cplx<float2> ldg_pair(const cplx<float>* p) {
  const float4 v = __ldg(reinterpret_cast<const float4*>(p));
  return mk(make_float2(v.x, v.z), make_float2(v.y, v.w));
}
__device__ __forceinline__ void st_pair(cplx<float>* p, cplx<float2> v) {
  *reinterpret_cast<float4*>(p) = make_float4(v.x.x, v.y.x, v.x.y, v.y.y);
}
__device__ __forceinline__ cplx<float2> zero_pair() { return mk(make_float2(0.f, 0.f), make_float2(0.f, 0.f)); }

// The compile-time plan when N > 0 (line stride LSC, CTA of NTB threads, by default
// L * ct_tpl<N>()), else the runtime plan P.
template <int DIR, int L, typename T, int N, class LD, class ST, int LSC = L, int NTB = 0>
__device__ __forceinline__ void fft_lines_n(const FftPlan& P, cplx<T>* s0, cplx<T>* s1, int LS,
                                            const cplx<T>* __restrict__ tw, LD ld, ST st) {
  if constexpr (N > 0) fft_lines_ct<DIR, L, T, N, LD, ST, LSC, NTB>(s0, s1, tw, ld, st);
  else fft_lines<DIR, L, T>(P, s0, s1, LS, tw, ld, st);
}

}  // namespace ffsgpu
