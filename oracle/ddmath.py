"""Double-double elementary functions for the oracle (test infrastructure only).

The reference's ETD3 phi-coefficients (src/time_step_functions/ETD.jl:181-191,
ETD1stand2ndO.jl:23,55-61) evaluate expm1 inside formulas that cancel catastrophically
when -c dt is just above the 1e-4 Taylor switch: an ulp of difference in expm1 becomes
~1e-9 relative in the coefficient. To compare two implementations at 1e-12, both must
feed those formulas the same doubles. This module evaluates expm1/exp (and the fused
multiply-add the reference's ``muladd`` compiles to) in double-double arithmetic and
rounds once, so the result is the correctly rounded value except in vanishingly rare
ties. The GPU engine runs the identical sequence of IEEE operations
(csrc/ffs_ddmath.cuh), so both sides produce the same bits.

Every function is elementwise on float64 numpy arrays; operation order is fixed and
must stay in step with the device code.

Methods: Veltkamp's splitting and Dekker's exact product (Dekker, Numer. Math. 18, 1971),
Knuth's exact sum (TAOCP vol. 2, section 4.2.2), double-double arithmetic as in Hida, Li
and Bailey's QD library (ARITH-15, 2001); exp/expm1 by k ln 2 argument reduction and a
double-double Taylor series.
"""
from __future__ import annotations

import numpy as np

_SPLIT = 134217729.0          # 2^27 + 1 (Veltkamp split)
LN2_HI = 0.6931471805599453   # ln 2 as a double-double
LN2_LO = 2.3190468138462996e-17
INV_LN2 = 1.4426950408889634
NTERMS = 27                   # Taylor terms; |x| <= 0.5 -> truncation < 1e-37 relative


def split(a):
    t = _SPLIT * a
    hi = t - (t - a)
    return hi, a - hi


def two_prod(a, b):
    p = a * b
    ah, al = split(a)
    bh, bl = split(b)
    e = (((ah * bh - p) + ah * bl) + al * bh) + al * bl
    return p, e


def two_sum(a, b):
    s = a + b
    bb = s - a
    return s, (a - (s - bb)) + (b - bb)


def quick_two_sum(a, b):
    s = a + b
    return s, b - (s - a)


def dd_add(ah, al, bh, bl):
    s1, s2 = two_sum(ah, bh)
    t1, t2 = two_sum(al, bl)
    s2 = s2 + t1
    s1, s2 = quick_two_sum(s1, s2)
    s2 = s2 + t2
    return quick_two_sum(s1, s2)


def dd_mul(ah, al, bh, bl):
    p, e = two_prod(ah, bh)
    e = e + (ah * bl + al * bh)
    return quick_two_sum(p, e)


def dd_div_d(ah, al, b):
    q1 = ah / b
    p1, p2 = two_prod(q1, b)
    s, e = two_sum(ah, -p1)
    e = e - p2
    e = e + al
    q2 = (s + e) / b
    return quick_two_sum(q1, q2)


def dd_mul_d(ah, al, b):
    p, e = two_prod(ah, b)
    e = e + al * b
    return quick_two_sum(p, e)


def fma(a, b, c):
    """a*b + c with one rounding (emulated; what Julia's muladd lowers to on FMA hardware)."""
    a, b, c = (np.asarray(v, dtype=np.float64) for v in (a, b, c))
    p, e = two_prod(a, b)
    sh, sl = dd_add(p, e, c, np.zeros_like(c))
    return sh


def _expm1_series(rh, rl):
    """expm1 of a double-double |r| <= 0.5 by its Taylor series, in double-double."""
    th, tl = rh, rl
    sh, sl = rh, rl
    for n in range(2, NTERMS + 1):
        th, tl = dd_mul(th, tl, rh, rl)
        th, tl = dd_div_d(th, tl, float(n))
        sh, sl = dd_add(sh, sl, th, tl)
    return sh, sl


def _exp_reduced(x):
    """exp(x) as (hi, lo, k): exp(x) = (hi + lo) * 2^k, |x - k ln2| <= ln2/2."""
    k = np.rint(x * INV_LN2)
    ph, pl = dd_mul_d(np.full_like(x, LN2_HI), np.full_like(x, LN2_LO), k)
    rh, rl = dd_add(x, np.zeros_like(x), -ph, -pl)
    eh, el = _expm1_series(rh, rl)
    h, l = dd_add(np.ones_like(x), np.zeros_like(x), eh, el)
    return h, l, k


def expm1(x):
    x = np.asarray(x, dtype=np.float64)
    xs = np.where(np.abs(x) <= 0.5, x, 0.0)
    small, _ = _expm1_series(xs, np.zeros_like(xs))
    xl = np.where((np.abs(x) > 0.5) & (x >= -40.0) & (x <= 700.0), x, 1.0)
    h, l, k = _exp_reduced(xl)
    h = np.ldexp(h, k.astype(np.int64))
    l = np.ldexp(l, k.astype(np.int64))
    big, _ = dd_add(h, l, np.full_like(x, -1.0), np.zeros_like(x))
    out = np.where(np.abs(x) <= 0.5, small, big)
    out = np.where(x < -40.0, -1.0, out)
    out = np.where(x > 700.0, np.inf, out)
    return out


def exp(x):
    x = np.asarray(x, dtype=np.float64)
    xs = np.where(np.abs(x) <= 0.5, x, 0.0)
    eh, el = _expm1_series(xs, np.zeros_like(xs))
    small, _ = dd_add(np.ones_like(x), np.zeros_like(x), eh, el)
    xl = np.where((np.abs(x) > 0.5) & (x >= -700.0) & (x <= 700.0), x, 1.0)
    h, l, k = _exp_reduced(xl)
    big = np.ldexp(h, k.astype(np.int64))
    out = np.where(np.abs(x) <= 0.5, small, big)
    out = np.where(x < -700.0, 0.0, out)
    out = np.where(x > 700.0, np.inf, out)
    return out
