// Double-double expm1 / exp / fma and the ETD phi-coefficients in a fixed order of
// IEEE round-to-nearest operations (no contraction into FMA).
//
// The reference's ETD coefficient formulas (ETD.jl:181-191, ETD1stand2ndO.jl:23,55-61)
// cancel catastrophically when -c dt is just above the 1e-4 Taylor switch, so any
// ulp-level difference in expm1, exp or in the operation order becomes ~1e-9 relative
// in the coefficients. Evaluating expm1/exp in double-double and rounding once gives the
// correctly rounded value (except in vanishingly rare ties), and writing every
// operation with __d*_rn pins the order, so the coefficients do not depend on the
// compiler. The same sequence of operations is used by the CPU oracle.
//
// The error-free transformations are the published ones: Veltkamp's splitting and
// Dekker's exact product (T. J. Dekker, "A floating-point technique for extending the
// available precision", Numer. Math. 18, 1971), Knuth's branch-free exact sum (D. E.
// Knuth, TAOCP vol. 2, section 4.2.2), and double-double addition, multiplication and
// renormalisation as in Hida, Li and Bailey's QD library ("Algorithms for quad-double
// precision floating point arithmetic", ARITH-15, 2001). exp/expm1 reduce the argument
// by k ln 2 (ln 2 held as a double-double) and sum the Taylor series in double-double.
#pragma once
#include <cuda_runtime.h>

namespace ffsgpu {
namespace dd {

__device__ __forceinline__ double A(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double S(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double M(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double D(double a, double b) { return __ddiv_rn(a, b); }

struct dd2 { double h, l; };

__device__ __forceinline__ void split(double a, double& hi, double& lo) {
  const double t = M(134217729.0, a);
  hi = S(t, S(t, a));
  lo = S(a, hi);
}
__device__ __forceinline__ dd2 two_prod(double a, double b) {
  const double p = M(a, b);
  double ah, al, bh, bl;
  split(a, ah, al);
  split(b, bh, bl);
  const double e = A(A(A(S(M(ah, bh), p), M(ah, bl)), M(al, bh)), M(al, bl));
  return {p, e};
}
__device__ __forceinline__ dd2 two_sum(double a, double b) {
  const double s = A(a, b);
  const double bb = S(s, a);
  return {s, A(S(a, S(s, bb)), S(b, bb))};
}
__device__ __forceinline__ dd2 quick_two_sum(double a, double b) {
  const double s = A(a, b);
  return {s, S(b, S(s, a))};
}
__device__ __forceinline__ dd2 add(dd2 a, dd2 b) {
  dd2 s = two_sum(a.h, b.h);
  dd2 t = two_sum(a.l, b.l);
  s.l = A(s.l, t.h);
  s = quick_two_sum(s.h, s.l);
  s.l = A(s.l, t.l);
  return quick_two_sum(s.h, s.l);
}
__device__ __forceinline__ dd2 mul(dd2 a, dd2 b) {
  dd2 p = two_prod(a.h, b.h);
  p.l = A(p.l, A(M(a.h, b.l), M(a.l, b.h)));
  return quick_two_sum(p.h, p.l);
}
__device__ __forceinline__ dd2 div_d(dd2 a, double b) {
  const double q1 = D(a.h, b);
  const dd2 p = two_prod(q1, b);
  dd2 s = two_sum(a.h, -p.h);
  s.l = S(s.l, p.l);
  s.l = A(s.l, a.l);
  const double q2 = D(A(s.h, s.l), b);
  return quick_two_sum(q1, q2);
}
__device__ __forceinline__ dd2 mul_d(dd2 a, double b) {
  dd2 p = two_prod(a.h, b);
  p.l = A(p.l, M(a.l, b));
  return quick_two_sum(p.h, p.l);
}

// a*b + c with one rounding (what Julia's muladd lowers to on FMA hardware)
__device__ __forceinline__ double fma_e(double a, double b, double c) {
  const dd2 p = two_prod(a, b);
  return add(p, dd2{c, 0.0}).h;
}

__device__ inline dd2 expm1_series(dd2 r) {
  dd2 t = r, s = r;
  for (int n = 2; n <= 27; ++n) {
    t = mul(t, r);
    t = div_d(t, (double)n);
    s = add(s, t);
  }
  return s;
}

// exp(x) = (h + l) * 2^k with |x - k ln2| <= ln2 / 2
__device__ inline dd2 exp_reduced(double x, double& k) {
  k = rint(M(x, 1.4426950408889634));
  const dd2 p = mul_d(dd2{0.6931471805599453, 2.3190468138462996e-17}, k);
  const dd2 r = add(dd2{x, 0.0}, dd2{-p.h, -p.l});
  const dd2 e = expm1_series(r);
  return add(dd2{1.0, 0.0}, e);
}

__device__ inline double expm1_cr(double x) {
  if (fabs(x) <= 0.5) return expm1_series(dd2{x, 0.0}).h;
  if (x < -40.0) return -1.0;
  if (x > 700.0) return INFINITY;
  double k;
  const dd2 e = exp_reduced(x, k);
  const int ki = (int)k;
  return add(dd2{ldexp(e.h, ki), ldexp(e.l, ki)}, dd2{-1.0, 0.0}).h;
}

__device__ inline double exp_cr(double x) {
  if (fabs(x) <= 0.5) return add(dd2{1.0, 0.0}, expm1_series(dd2{x, 0.0})).h;
  if (x < -700.0) return 0.0;
  if (x > 700.0) return INFINITY;
  double k;
  const dd2 e = exp_reduced(x, k);
  return ldexp(e.h, (int)k);
}

}  // namespace dd

// ETD phi-coefficients: u' = E u + A N + B fm1 + C fm2 for stage 1 (ETD1), 2 (ETD2),
// 3 (ETD3). Each expression follows the reference's left-to-right evaluation; muladd
// is the emulated single-rounding fma.
// CR = true: exp/expm1 correctly rounded (double-double), for bit parity of the FP64
// form. CR = false: CUDA's FP64 exp/expm1 (within an ulp or two), for the FP32 form,
// whose coefficients are rounded to FP32 afterwards; the formulas are the same.
template <bool CR>
__device__ inline double etd_exp(double x) { return CR ? dd::exp_cr(x) : exp(x); }
template <bool CR>
__device__ inline double etd_expm1(double x) { return CR ? dd::expm1_cr(x) : expm1(x); }

template <bool CR = true>
__device__ inline void etd_coeffs_exact(double c, double dt, double dt2, double dt3, int stage, double& E,
                                        double& Ac, double& Bc, double& Cc) {
  using namespace dd;
  const double cdt = M(c, dt);
  E = etd_exp<CR>(cdt);
  const bool test = M(-c, dt) <= 1e-4;
  const bool inf = (c == -INFINITY);
  if (stage == 1) {   // ETD1stand2ndO.jl:12-26
    const double cdt2 = M(cdt, dt), c2dt3 = M(cdt2, cdt), c3dt4 = M(c2dt3, cdt);
    if (inf) Ac = 0.0;
    else if (test) Ac = A(A(A(dt, M(0.5, cdt2)), D(c2dt3, 6.0)), D(c3dt4, 24.0));
    else Ac = D(etd_expm1<CR>(cdt), c);
    Bc = 0.0; Cc = 0.0;
    return;
  }
  if (stage == 2) {   // ETD1stand2ndO.jl:37-66
    const double cp2 = M(c, c), cdtp2 = M(cdt, dt), c2dtp3 = M(cdtp2, cdt), c3dtp4 = M(c2dtp3, cdt);
    const double em = etd_expm1<CR>(cdt), c2dt2 = M(M(c, c), dt2);
    const double dtp2 = M(dt, dt), dtp3 = M(dtp2, dt), dtp4 = M(dtp3, dt);
    if (inf) { Ac = 0.0; Bc = 0.0; }
    else if (test) {
      Ac = A(A(A(A(A(A(dt, D(cdtp2, 2.0)), D(c2dtp3, 6.0)), D(c3dtp4, 24.0)), D(dtp2, M(2.0, dt2))),
               D(M(c, dtp3), M(6.0, dt2))),
             D(M(cp2, dtp4), M(24.0, dt2)));
      Bc = S(S(-D(dtp2, M(2.0, dt2)), D(M(c, dtp3), M(6.0, dt2))), D(M(cp2, dtp4), M(24.0, dt2)));
    } else {
      Ac = D(S(em, M(c, S(dt, M(dt2, em)))), c2dt2);
      Bc = D(S(cdt, em), c2dt2);
    }
    Cc = 0.0;
    return;
  }
  // ETD3 (ETD.jl:152-227)
  const double d23 = A(dt2, dt3);
  const double tdt2 = M(2.0, dt2);
  const double a0 = D(M(dt, A(A(M(M(2.0, dt), dt), M(M(6.0, dt2), d23)), M(M(3.0, dt), A(tdt2, dt3)))),
                      M(M(6.0, dt2), d23));
  const double a1 = D(M(M(dt, dt), A(A(M(dt, dt), M(M(6.0, dt2), d23)), M(M(2.0, dt), A(tdt2, dt3)))),
                      M(M(12.0, dt2), d23));
  const double a2 = D(M(M(M(dt, dt), dt), A(M(M(4.0, dt2), d23), M(dt, A(tdt2, dt3)))), M(M(24.0, dt2), d23));
  const double a3 = D(M(M(M(dt, dt), dt), dt), 24.0);
  const double b0 = -D(M(M(dt, dt), A(M(2.0, dt), M(3.0, d23))), M(6.0, M(dt2, dt3)));
  const double b1 = -D(M(M(M(dt, dt), dt), A(dt, M(2.0, d23))), M(12.0, M(dt2, dt3)));
  const double b2 = -D(M(M(M(M(dt, dt), dt), dt), d23), M(24.0, M(dt2, dt3)));
  const double c0 = D(M(M(dt, dt), A(M(2.0, dt), M(3.0, dt2))), M(M(6.0, dt3), d23));
  const double c1 = D(M(M(M(dt, dt), dt), A(dt, M(2.0, dt2))), M(M(12.0, dt3), d23));
  const double c2 = D(M(M(M(M(dt, dt), dt), dt), dt2), M(M(24.0, dt3), d23));
  const double e1 = A(M(dt, dt), M(dt, A(tdt2, dt3)));
  const double e2 = M(dt2, d23);
  const double e3 = M(2.0, dt);
  const double e4 = A(tdt2, dt3);
  const double e5 = M(dt, A(A(dt, dt2), dt3));
  const double e6 = d23;
  const double e7 = M(dt2, dt3);
  const double e8 = M(dt, A(dt, dt2));
  const double e9 = M(dt3, d23);
  const double l1 = c, l2 = M(l1, l1), l3 = M(l2, l1);
  if (inf) { Ac = Bc = Cc = 0.0; return; }
  if (test) {
    Ac = fma_e(a1, l1, fma_e(a2, l2, fma_e(a3, l3, a0)));
    Bc = fma_e(b1, l1, fma_e(b2, l2, b0));
    Cc = fma_e(c1, l1, fma_e(c2, l2, c0));
  } else {
    const double em = etd_expm1<CR>(M(l1, dt));
    Ac = D(S(S(M(2.0, em), M(l2, S(e1, M(e2, em)))), M(l1, S(e3, M(e4, em)))), M(l3, e2));
    Bc = D(A(S(M(e5, l2), M(2.0, em)), M(l1, S(e3, M(e6, em)))), M(l3, e7));
    Cc = D(S(S(M(2.0, em), M(e8, l2)), M(l1, S(e3, M(dt2, em)))), M(l3, e9));
  }
}

}  // namespace ffsgpu
