"""Scales.txt and Numbers.txt (writeheader / writestats / stats, src/stats.jl:9-62, 64-165)
from the engine's stats records.

Every record holds the Stats.txt columns, then the integral-length plane sums
(integral_lenght_x/y/z, stats.jl:952-980: for each velocity component the kx = 0, ky = 0
and kz = 0 plane sums of |u|^2, the last two with the (1 + [kx > 0]) weight) and the
derivative means du1/dy, du1/dx, du2/dy, du2/dx (dy/dx_squared_mean, stats.jl:334-400).
The length scales, time scales and Reynolds/Froude numbers follow from those in FP64.
"""
from __future__ import annotations

import math

SCALES_HEADER = ("iteration,time,Lk,Lt,lamg,laml,lamt,Lhh,Lvv,Lhv,Lvh,lam12,lam21,L11,L12,L13,L21,L22,L23,"
                 "L31,L32,L33")
NUMBERS_HEADER = "iteration,time,Reh,Reh1,Relamg,Relaml,Relamt,Relamg1,Relaml1,Relamt1"


def scales_header(density: bool) -> str:
    return SCALES_HEADER + (",Lb,Lo,Lom,Tk,Tt,Thh,Tb,Tbm" if density else ",Tk,Tt,Thh")


def numbers_header(density: bool) -> str:
    return NUMBERS_HEADER + (",Reb,Rebm,Frh,Frh1" if density else "")


def _div(a, b):
    try:
        return a / b
    except ZeroDivisionError:
        return math.copysign(math.inf, a) if a != 0 else math.nan


def _sqrt(x):
    return math.sqrt(x) if x >= 0 else math.nan


def scales_numbers(rec, header: list[str], ncols_stats: int, nu: float, lx: float, ly: float, lz: float,
                   density: bool = False, n2: float = 0.0) -> tuple[list[float], list[float]]:
    """(Scales row, Numbers row) without iteration and time, for one record.

    n2 = g_z * drho/dz (calculate_N, density_stratification_types.jl:32-34). For the
    velocity-only case the reference writes six numbers under an eight-name header
    (stats.jl:160-162); the rows here are the reference's.
    """
    col = {name: i for i, name in enumerate(header)}
    u1p2, u2p2, u3p2 = rec[col["u1p2"]], rec[col["u2p2"]], rec[col["u3p2"]]
    k, tdiss = rec[col["k"]], rec[col["tdiss"]]
    r = [rec[ncols_stats + i] for i in range(9)]
    du1dyp2, du1dxp2, du2dyp2, du2dxp2 = (rec[ncols_stats + 9 + i] for i in range(4))
    lens3 = (lx, ly, lz)
    up2 = (u1p2, u2p2, u3p2)
    L = [_div(lens3[p] * r[3 * c + p] * math.pi, up2[c]) for c in range(3) for p in range(3)]
    L11, L12, L13, L21, L22, L23, L31, L32, L33 = L
    uh = _sqrt((u1p2 + u2p2) / 2)
    urms = _sqrt((u1p2 + u2p2 + u3p2) / 3)
    lam12 = _sqrt(_div(2 * u1p2, du1dyp2))
    lam21 = _sqrt(_div(2 * u2p2, du2dxp2))
    Lhh = (L11 + L22) / 2
    Thh = _div(Lhh, urms)
    laml = _sqrt(_div(2 * (u1p2 + u2p2), du1dxp2 + du2dyp2))
    lamt = _sqrt(_div(2 * (u1p2 + u2p2), du1dyp2 + du2dxp2))
    Lhv = (L13 + L23) / 2
    Lvv = L33
    Lvh = (L31 + L32) / 2
    Lt = _div(_sqrt(k * k * k), tdiss)
    Tt = _div(k, tdiss)
    Lk = _sqrt(_sqrt(_div(nu * nu * nu, tdiss)))
    Tk = _sqrt(_div(nu, tdiss))
    lamg = _sqrt(_div(15 * nu, tdiss)) * urms
    lensv = [Lk, Lt, lamg, laml, lamt, Lhh, Lvv, Lhv, Lvh, lam12, lam21, L11, L12, L13, L21, L22, L23, L31, L32, L33]

    def p43(a, b):
        q = _div(a, b)
        return q ** (4 / 3) if q >= 0 else math.nan

    Reh = _div(uh * Lhh, nu)
    Reh1 = p43(Lhh, Lk)
    Relg, Relg1 = _div(urms * lamg, nu), p43(lamg, Lk)
    Rell, Rell1 = _div(urms * laml, nu), p43(laml, Lk)
    Relt, Relt1 = _div(urms * lamt, nu), p43(lamt, Lk)
    if density:
        Nb = _sqrt(n2)
        Lb = _div(2 * math.pi * urms, Nb)
        Lo = _sqrt(_div(tdiss, Nb * Nb * Nb))
        Lom = _sqrt(_div(tdiss, Nb * Nb * Nb / (8 * math.pi * math.pi * math.pi)))
        Tb = _div(2 * math.pi, Nb)
        Tbm = _div(1.0, Nb)
        Reb, Rebm = p43(Lo, Lk), p43(Lom, Lk)
        Frh = _div(2 * math.pi * uh, Nb * Lhh)
        Frh1 = _div(Lhv, Lhh)
        return lensv + [Lb, Lo, Lom, Tk, Tt, Thh, Tb, Tbm], [Reh, Reh1, Relg, Rell, Relt, Relg1, Rell1, Relt1, Reb,
                                                               Rebm, Frh, Frh1]
    return lensv + [Tk, Tt, Thh], [Reh, Reh1, Rell, Relt, Rell1, Relt1]
