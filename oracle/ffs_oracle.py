"""FP64 CPU restatement of FluidFlowSimulation.jl's solver step.

TEST INFRASTRUCTURE ONLY. This module is the checker that the GPU engine is compared
against; it is never part of the product path. It restates, operation for operation,
the reference's Julia code for one time step (``advance_in_time!``) and everything it
calls. Citations are ``file:line`` inside the reference project (``src/...``).

Parity status: the reference is pure Julia and needs Julia + FFTW, neither of which
exists in this environment, and its only test is a placeholder (``test/runtests.jl:5``).
This restatement is therefore pinned by analytic known-answer tests (Taylor-Green
invariants, exact linear decay under ETD, divergence-free projection, energy budget,
forcing power) rather than by reference outputs. FFTW is replaced by pocketfft
(``scipy.fft``); both are FP64 FFTs accurate to ~1e-16 relative.

Conventions (same memory order as the reference's column-major Julia arrays):
  physical arrays:  real  [z, y, x]           (x fastest)
  spectral arrays:  complex [z, y, kx], kx in 0..nx/2 (half spectrum), x fastest
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass, field

import numpy as np
import scipy.fft as sfft

from . import ddmath as dd

_WORKERS = int(os.environ.get("FFS_ORACLE_WORKERS", os.cpu_count() or 1))


# ----------------------------------------------------------------------------------
# Grid tables — src/Globals.jl
# ----------------------------------------------------------------------------------

def rfftfreq(n: int, s: float) -> np.ndarray:
    """``rfftfreq`` of ``src/Globals.jl:95-97``: ``[(n/2 - i)/s for i = n/2:-1:0]``."""
    i = np.arange(n / 2, -1.0, -1.0)
    return (n / 2 - i) / s


def fftfreq(n: int, s: float) -> np.ndarray:
    """``fftfreq`` of ``src/Globals.jl:99-104`` (Nyquist negative for even n)."""
    if n % 2 == 0:
        a = (n / 2 - np.arange(n / 2, 0.0, -1.0)) / s
        b = -np.arange(n / 2, 0.0, -1.0) / s
        return np.concatenate([a, b])
    a = (n / 2 - np.arange(n / 2, -0.5, -1.0)) / s
    b = -np.arange((n - 1) / 2, 0.0, -1.0) / s
    return np.concatenate([a, b])


@dataclass
class Grid:
    """Wavenumber tables, dealias mask and retained ranges (``src/Globals.jl:106-171``)."""

    nx: int
    ny: int
    nz: int
    lx: float = 1.0
    ly: float = 1.0
    lz: float = 1.0
    cutoff: float = 2.0 / 3.0

    def __post_init__(self):
        self.nxh = self.nx // 2 + 1
        self.kx = rfftfreq(self.nx, self.lx)            # Globals.jl:119
        self.ky = fftfreq(self.ny, self.ly)             # Globals.jl:120
        self.kz = fftfreq(self.nz, self.lz)             # Globals.jl:121
        c = self.cutoff
        cx = (c * self.kx[-1]) ** 2                     # Globals.jl:136
        cy = (c * np.max(np.abs(self.ky))) ** 2         # Globals.jl:137
        cz = (c * np.max(np.abs(self.kz))) ** 2         # Globals.jl:138
        KX = self.kx[None, None, :]
        KY = self.ky[None, :, None]
        KZ = self.kz[:, None, None]
        # DEALIAS[i,j,k] = kx^2 > cx | ky^2 > cy | kz^2 > cz   (Globals.jl:142)
        self.dealias = (KX ** 2 > cx) | (KY ** 2 > cy) | (KZ ** 2 > cz)
        self.keep = ~self.dealias
        self.KX, self.KY, self.KZ = KX, KY, KZ
        # K2 = muladd(KX,KX, muladd(KY,KY,KZ*KZ))   (ETD.jl:66)
        self.K2 = KX * KX + (KY * KY + KZ * KZ)
        self.N = self.nx * self.ny * self.nz
        # 1D spectrum bins (Globals.jl:144-152, spec.jl:424-450)
        self.KH = self.kx if self.kx[1] >= self.ky[1] else rfftfreq(self.ny, self.ly)
        self.MAXDKH = self.KH[1]
        self.KRZ = rfftfreq(self.nz, self.lz)
        self.DKZ = self.KRZ[1]
        # weight for the Hermitian half spectrum: 1 + (i > 1) (stats.jl:301)
        self.w = np.where(np.arange(self.nxh) > 0, 2.0, 1.0)[None, None, :]

    # --- transforms (utils.jl:101-106; FluidFields real!) ---------------------------------
    def myfourier(self, phys: np.ndarray) -> np.ndarray:
        """Forward: unnormalised r2c, zero the DEALIAS modes, times 1/(nx ny nz)."""
        c = sfft.rfftn(phys, axes=(-3, -2, -1), workers=_WORKERS)
        c[..., self.dealias] = 0.0
        c *= 1.0 / self.N
        return c

    def real(self, spec: np.ndarray) -> np.ndarray:
        """Inverse: unnormalised c2r (FFTW brfft semantics)."""
        return sfft.irfftn(spec, s=(self.nz, self.ny, self.nx), axes=(-3, -2, -1),
                           norm="forward", workers=_WORKERS)

    def project(self, v: np.ndarray) -> np.ndarray:
        """``pressure_projection!`` (models.jl:443-456): v - k (k.v)/k^2, k=0 untouched."""
        kd = self.KX * v[0] + self.KY * v[1] + self.KZ * v[2]
        with np.errstate(divide="ignore", invalid="ignore"):
            p1 = -kd / self.K2
        p1[0, 0, 0] = 0.0
        return np.stack([p1 * self.KX + v[0], p1 * self.KY + v[1], p1 * self.KZ + v[2]])


# ----------------------------------------------------------------------------------
# Parameters — src/simulationtypes.jl:242-365 (in-scope keys only)
# ----------------------------------------------------------------------------------

def _num(s: str) -> float:
    """Parse a `global` numeric value (the reference runs ``eval(Meta.parse(...))``).

    Supports plain numbers, ``Inf`` and products/quotients with ``π``/``pi`` such as
    ``2π`` or ``2pi/128``.
    """
    import re
    t = s.strip().replace("π", "pi")
    t = re.sub(r"(\d)\s*pi", r"\1*pi", t)
    return float(eval(t, {"__builtins__": {}}, {"pi": math.pi, "Inf": math.inf}))


@dataclass
class Params:
    nx: int = 32
    ny: int = 32
    nz: int = 32
    lx: float = 1.0
    ly: float = 1.0
    lz: float = 1.0
    nu: float = 0.0
    cutoff: float = 2.0 / 3.0
    integrator: str = "ETD3rdO"          # or "Adams_Bashforth3rdO"
    variable_dt: bool = True
    cfl: float = 0.18
    dt: float = 0.0
    hv: bool = False
    hv_nu: float = 0.0
    hv_m: int = 2
    hv_kind: str = "power"               # "power" (HyperViscosity) or "barrier" (SpectralBarrier)
    hv_initk: float = 0.0
    hv_endk: float = 0.0
    rho_hv: str = ""                     # densityHyperViscosity: "", "power", "barrier"
    rho_hv_nu: float = 0.0
    rho_hv_m: int = 2
    rho_hv_initk: float = 0.0
    rho_hv_endk: float = 0.0
    les: bool = False
    les_model: str = "Smagorinsky"       # Smagorinsky, Vreman, productionViscosity, Silvis, stableNonLinear
    smag_c: float = 0.17                 # the model's constant c
    les_cp: float = 5.0                  # silvisPConstant
    les_test_width: float = 0.0          # dynamicSmagorinsky: TestFilterWidth (default 2 filterWidth)
    les_cmin: float = 0.0                # dynamicSmagorinsky: cmin
    les_dynp: str = ""                   # "dynamicSandP" / "piomelliSandP": the dynamic P tensor term
    sandp_cb: float = 0.0                # SandP: pConstant (0: no P term)
    rho_les: str = ""                    # LES of the density / scalar: "", "eddy", "vorticity"
    rho_les_c: float = 0.0               # densityVorticityCoefficient / scalarVorticityCoefficient
    filter_width: float | None = None
    scalar: bool = False                 # passiveScalar (simulationtypes.jl:198-213, :320-352)
    scalar_pr: float = 1.0
    scalar_gradient: float = 0.0
    scalar_dir: int = 2
    density: bool = False
    density_pr: float = 1.0
    density_gradient: float = 0.0
    gravity: float = 0.0                 # zAcceleration / referenceDensity
    gravity_dir: int = 2                 # 0 x, 1 y, 2 z
    forcing: bool = False
    forcing_power: float = 0.1
    forcing_kf: float = 2.5
    # the reference's kz = 0 plane forcing (forcing_types.jl:335-450): rfForcing, cRfForcing, QfForcing
    plane_forcing: str = ""
    pf_tf: float = 0.0                   # TF
    pf_alpha: float = 0.0                # alphac
    pf_kf: float = 0.0                   # kf
    pf_zf_tanh: bool = False             # Zf tanh (else cutoff)
    pf_qp: float = 0.0                   # alveliusP
    pf_qc: float = 0.0                   # alveliusC
    pf_qkf: float = 0.0                  # alveliusKf
    dt_stat: int = 1
    dt_spec: int = 1
    spec_fil: float = 0.0                # specFil: filtered stats and spectra (0: off)
    write_time: int = 1 << 30
    start: int = 0
    start_time: float = 0.0
    reference_cfl_slot: bool = True

    @property
    def fil_d2(self) -> float:
        """SPEC_FIL_D2 = (2 pi LX nf / NRX)^2 (Globals.jl:173-178); STAT_FIL = fil_d2 != 0."""
        return (2 * math.pi * self.lx * self.spec_fil / self.nx) ** 2 if self.spec_fil else 0.0

    @classmethod
    def from_global(cls, d: dict) -> "Params":
        """Mirror ``parameters(d)`` (simulationtypes.jl:242-365) for the in-scope keys."""
        p = cls()
        p.nx, p.ny, p.nz = int(d["nx"]), int(d["ny"]), int(d["nz"])
        p.lx, p.ly, p.lz = _num(d["xDomainSize"]), _num(d["yDomainSize"]), _num(d["zDomainSize"])
        p.nu = _num(d["kinematicViscosity"])
        if "cutoff" in d:
            p.cutoff = _num(d["cutoff"])
        p.start = int(d.get("start", 0))
        p.start_time = float(d.get("startTime", 0.0))
        p.dt_stat = int(d["dtStat"])
        p.dt_spec = int(d["dtSpec"])                       # KeyError like :262
        if "specFil" in d:                                 # Globals.jl:173-178
            p.spec_fil = float(d["specFil"])
        p.write_time = int(d["writeTime"])
        p.integrator = d.get("velocityTimeStep", "ETD3rdO")
        p.variable_dt = d.get("variableTimestepFlag", "true").strip().lower() == "true"
        p.cfl = float(d.get("cfl", 0.18))
        p.dt = _num(d["dt"]) if "dt" in d else 0.0
        kxm = (p.nx // 2) / p.lx                          # KX[end]
        if d.get("hyperViscosity") == "spectralBarrier":   # simulationtypes.jl:294-297
            p.hv = True
            p.hv_kind = "barrier"
            p.hv_initk = float(d["initk"]) if "initk" in d else p.cutoff * 2 * kxm / 3
            p.hv_endk = float(d["endk"]) if "endk" in d else math.sqrt(p.cutoff * 3) * kxm
        elif "hyperViscosity" in d:
            p.hv = True
            p.hv_nu = float(d["hyperViscosityCoefficient"])
            p.hv_m = int(d.get("hyperViscosityM", 2))
        if "densityHyperViscosity" in d and "densityStratification" in d:   # density_stratification_types.jl:137-148
            if d["densityHyperViscosity"] == "spectralBarrier":
                p.rho_hv = "barrier"
                p.rho_hv_initk = float(d["densityInitk"]) if "densityInitk" in d else p.cutoff * 2 * kxm / 3
                p.rho_hv_endk = float(d["densityEndk"]) if "densityEndk" in d else math.sqrt(p.cutoff * 3) * kxm
            else:
                p.rho_hv = "power"
                p.rho_hv_nu = float(d["densityHyperViscosityCoefficient"])
                p.rho_hv_m = int(d.get("densityHyperViscosityM", 2))
        if "lesModel" in d:
            p.set_les(d)
        if "densityStratification" in d:
            p.density = True
            p.density_pr = _num(d["Pr"])
            p.density_gradient = _num(d["densityGradient"])
            p.gravity = _num(d["zAcceleration"]) / _num(d["referenceDensity"])
            p.gravity_dir = {"x": 0, "y": 1, "z": 2}[d.get("gravityDirection", "z")]
        if "densityLesModel" in d and "densityStratification" in d:   # density_stratification_types.jl:176-185
            if "lesModel" not in d:
                raise ValueError("densityLesModel without lesModel is not restated")
            vort = d["densityLesModel"] == "vorticityDiffusion"
            p.rho_les = "vorticity" if vort else "eddy"
            p.rho_les_c = float(d.get("densityVorticityCoefficient", "0.1")) if vort else 0.0
        if "passiveScalar" in d:
            if "densityStratification" in d:
                raise ValueError("a passive scalar together with density stratification is not restated")
            if "lesModel" in d:                            # simulationtypes.jl:334-346
                vort = d.get("scalarLesModel") == "vorticityDiffusion"
                p.rho_les = "vorticity" if vort else "eddy"
                p.rho_les_c = float(d.get("scalarVorticityCoefficient", "1.0")) if vort else 0.0
            p.scalar = True
            p.scalar_pr = _num(d["scalarPr"])
            p.scalar_gradient = _num(d["scalarGradient"])
            p.scalar_dir = {"x": 0, "y": 1, "z": 2}[d.get("scalarDirection", "z")]
        if d.get("forcing") in PLANE_KINDS:
            p.plane_forcing = d["forcing"]
            p.pf_kf = float(d["kf"])
            if p.plane_forcing == "QfForcing":
                p.pf_qp, p.pf_qc, p.pf_qkf = (float(d[k]) for k in ("alveliusP", "alveliusC", "alveliusKf"))
            else:
                p.pf_tf, p.pf_alpha = float(d["TF"]), float(d["alphac"])
                p.pf_zf_tanh = d.get("Zf", "cutoff") != "cutoff"
        if d.get("forcing") == "isotropicBand":
            p.forcing = True
            p.forcing_power = _num(d.get("forcingPower", "0.1"))
            p.forcing_kf = _num(d.get("forcingKf", "2.5"))
        if "referenceCflSlot" in d:
            p.reference_cfl_slot = d["referenceCflSlot"].strip().lower() == "true"
        return p

    def set_les(self, d: dict) -> None:
        """The pointwise LES models of ``les_types`` (les_types.jl:360-395): the model's
        constant and filter width with the reference's defaults; SandP adds the P tensor
        to an eddy-viscosity model (sLesModel)."""
        m = d["lesModel"]
        base = m
        if m == "SandP" and d.get("sLesModel") in ("dynamicSmagorinsky", "piomelliSmagorinsky"):
            # SandP on a dynamic model (les_types.jl:401-416): beta = cb D^2 (les_real_calc.jl:57-58)
            self.sandp_cb = _num(d.get("pConstant", "0.09"))
            m = base = d["sLesModel"]
        if m in ("dynamicSandP", "piomelliSandP"):         # les_types.jl:426-455
            base = d["sLesModel"]
            if base not in ("dynamicSmagorinsky", "piomelliSmagorinsky"):
                raise ValueError(f"LES model {m} / {base} is not restated")
            self.les_dynp = m
            m = base
        if m in ("dynamicSmagorinsky", "piomelliSmagorinsky"):   # les_types.jl:388-397
            self.les = True
            self.les_model = m
            dx = (self.lx * 2 * math.pi / self.nx) / self.cutoff
            self.filter_width = _num(d["filterWidth"]) if "filterWidth" in d else dx
            self.les_test_width = (_num(d["TestFilterWidth"]) if "TestFilterWidth" in d
                                   else 2 * self.filter_width)
            self.les_cmin = float(d["cmin"]) if "cmin" in d else 0.0
            return
        if m == "SandP":
            base = d["sLesModel"]
            self.sandp_cb = _num(d.get("pConstant", "0.09"))
        consts = {"Smagorinsky": ("smagorinskyConstant", 0.17), "Vreman": ("vremanConstant", 0.032),
                  "productionViscosity": ("productionConstant", 0.1 if m == "SandP" else 0.4),
                  "Silvis": ("silvisConstant", math.sqrt(0.17)), "stableNonLinear": ("nlConstant", 0.1)}
        if base not in consts or (m == "SandP" and base in ("Silvis", "stableNonLinear")):
            raise ValueError(f"LES model {m} / {base} is not restated")
        key, dflt = consts[base]
        self.les = True
        self.les_model = base
        self.smag_c = _num(d[key]) if key in d else dflt
        if base == "Silvis":
            self.les_cp = _num(d["silvisPConstant"]) if "silvisPConstant" in d else 5.0
        dx = (self.lx * 2 * math.pi / self.nx) / self.cutoff
        if m == "SandP" and base == "Smagorinsky":
            dx = 2 * dx                                         # les_types.jl:395
        self.filter_width = _num(d["filterWidth"]) if "filterWidth" in d else dx

    @property
    def fld(self) -> bool:
        """A transported scalar field rides beside the velocity (density or passive scalar)."""
        return self.density or self.scalar

    @property
    def fld_grad(self) -> float:
        return self.density_gradient if self.density else self.scalar_gradient

    @property
    def fld_dir(self) -> int:
        return self.gravity_dir if self.density else self.scalar_dir

    @property
    def ab3(self) -> bool:
        """An explicit integrator (Adams_Bashforth3rdO or Euller): the viscosity, the
        hyperviscosity and the scalar's diffusion are terms of the right-hand side
        (is_implicit, time_step_functions.jl:5-7; models.jl:296-326,356-361)."""
        return self.integrator in ("Adams_Bashforth3rdO", "Euller")


# ----------------------------------------------------------------------------------
# Time integrators — src/time_step_functions/*.jl
# ----------------------------------------------------------------------------------

class AB3:
    """Adams-Bashforth 3 (Adams_Bashforth.jl:1-128) with the Euler/AB2 start-up."""

    def __init__(self, adaptive: bool, idt: float):
        self.adaptive = adaptive
        self.dt = self.dt2 = self.dt3 = idt            # Adams_Bashforth.jl:13-23
        self.iteration = 0
        self.fm1 = None
        self.fm2 = None

    def initialize(self, rhs, dt_now):
        """Adams_Bashforth.jl:28-35: fm1 = fm2 = rhs, dt history = current dt."""
        self.fm1 = rhs.copy()
        self.fm2 = rhs.copy()
        self.dt = dt_now
        self.dt2 = self.dt
        self.dt3 = self.dt

    def set_dt(self, dt):
        """Adams_Bashforth.jl:37-47 (adaptive only)."""
        if not self.adaptive:
            return
        if self.iteration == 0:
            self.dt3 = self.dt2 = self.dt = dt / 2
        else:
            self.dt3 = self.dt2
            self.dt2 = self.dt
            self.dt = dt

    def coefficients(self):
        """Adaptive formulas (Adams_Bashforth.jl:49-89); fixed dt: 23/12, -16/12, 5/12 dt."""
        dt, dt2, dt3 = self.dt, self.dt2, self.dt3
        if not self.adaptive:
            return 23 * dt / 12, -16 * dt / 12, 5 * dt / 12
        At = (1.0 + (dt * (2 * dt + 6 * dt2 + 3 * dt3)) / (6 * dt2 * (dt2 + dt3))) * dt
        Bt = (-dt * dt * (2 * dt + 3 * dt2 + 3 * dt3) / (6 * dt2 * dt3 * (dt + dt2))) * (dt + dt2)
        Ct = (dt * dt * (2 * dt + 3 * dt2) / (6 * dt3 * (dt + dt2 + dt3) * (dt2 + dt3))) * (dt + dt2 + dt3)
        return At, Bt, Ct

    def step(self, u, rhs, explicit=None):
        """Adams_Bashforth.jl:102-128 (+ fix_fm2! at the second call, ETD.jl:130-140)."""
        self.iteration += 1
        if self.iteration == 2:
            self.fm2 = -(self.dt3 + self.dt2) * (rhs - self.fm1) / self.dt2 + rhs
        At, Bt, Ct = self.coefficients()
        unew = At * rhs + (Bt * self.fm1 + (Ct * self.fm2 + u))
        self.fm2 = self.fm1
        self.fm1 = rhs.copy()
        return unew


class Euler:
    """Euller (Euller.jl:1-25): u = dt rhs + u, dt as set_dt! gives it (no start-up
    halving). The reference builds it as Euller{variableTimeStep,idt}, one type parameter
    more than the struct declares (simulationtypes.jl:312-313), so this is the intended
    integrator."""

    def __init__(self, adaptive: bool, idt: float):
        self.adaptive = adaptive
        self.dt = self.dt2 = self.dt3 = idt
        self.iteration = 0

    def initialize(self, rhs, dt_now):
        self.dt = dt_now

    def set_dt(self, dt):
        if self.adaptive:
            self.dt = dt

    def step(self, u, rhs, explicit=None):
        self.iteration += 1
        return self.dt * rhs + u


class ETD3:
    """Exponential time differencing, 3rd order (ETD.jl:3-261, ETD1stand2ndO.jl:1-66)."""

    def __init__(self, adaptive: bool, idt: float, c: np.ndarray):
        self.adaptive = adaptive
        self.dt = self.dt2 = self.dt3 = idt            # ETD.jl:33-36
        self.iteration = 0
        self.c = c                                      # c = -nu k^2 (- nuh k^2M)
        self.fm1 = None
        self.fm2 = None
        self.At = self.Bt = self.Ct = None

    def set_dt(self, dt):
        """ETD.jl:110-114 — rotates on every call when adaptive."""
        if not self.adaptive:
            return
        self.dt3 = self.dt2
        self.dt2 = self.dt
        self.dt = dt

    def initialize(self, rhs, dt_now):
        """ETD.jl:99-108."""
        self.fm1 = rhs.copy()
        self.fm2 = rhs.copy()
        self.dt = dt_now
        self.dt2 = self.dt
        self.dt3 = self.dt
        self.set_dt(self.dt)
        if not self.adaptive:
            self.set_ABCt()

    def set_ABCt(self):
        """ETD.jl:142-227 (Taylor branch when -c dt <= 1e-4, zero when c == -Inf)."""
        l1 = self.c
        dt, dt2, dt3 = self.dt, self.dt2, self.dt3
        # left-to-right evaluation exactly as written in ETD.jl:198-227 / 164-191
        a0 = (dt * (2 * dt * dt + 6 * dt2 * (dt2 + dt3) + 3 * dt * (2 * dt2 + dt3))) / (6 * dt2 * (dt2 + dt3))
        a1 = (dt * dt * (dt * dt + 6 * dt2 * (dt2 + dt3) + 2 * dt * (2 * dt2 + dt3))) / (12 * dt2 * (dt2 + dt3))
        a2 = (dt * dt * dt * (4 * dt2 * (dt2 + dt3) + dt * (2 * dt2 + dt3))) / (24 * dt2 * (dt2 + dt3))
        a3 = dt * dt * dt * dt / 24
        b0 = -((dt * dt * (2 * dt + 3 * (dt2 + dt3))) / (6 * (dt2 * dt3)))
        b1 = -(((dt * dt * dt * (dt + 2 * (dt2 + dt3)))) / (12 * (dt2 * dt3)))
        b2 = -((dt * dt * dt * dt * (dt2 + dt3)) / (24 * (dt2 * dt3)))
        c0 = (dt * dt * (2 * dt + 3 * dt2)) / (6 * dt3 * (dt2 + dt3))
        c1 = (dt * dt * dt * (dt + 2 * dt2)) / (12 * dt3 * (dt2 + dt3))
        c2 = (dt * dt * dt * dt * dt2) / (24 * dt3 * (dt2 + dt3))
        e1 = dt * dt + dt * (2 * dt2 + dt3)
        e2 = dt2 * (dt2 + dt3)
        e3 = 2 * dt
        e4 = 2 * dt2 + dt3
        e5 = dt * (dt + dt2 + dt3)
        e6 = dt2 + dt3
        e7 = dt2 * dt3
        e8 = dt * (dt + dt2)
        e9 = dt3 * (dt2 + dt3)
        l2 = l1 * l1
        l3 = l2 * l1
        test = (-l1) * dt <= 1e-4
        with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
            em = dd.expm1(l1 * dt)
            # muladd -> single-rounding fma (dd.fma) in the Taylor branch
            At = np.where(test, dd.fma(a1, l1, dd.fma(a2, l2, dd.fma(a3, l3, a0))),
                          ((2 * em - l2 * (e1 - e2 * em)) - l1 * (e3 - e4 * em)) / (l3 * e2))
            Bt = np.where(test, dd.fma(b1, l1, dd.fma(b2, l2, b0)),
                          ((e5 * l2 - 2 * em) + l1 * (e3 - e6 * em)) / (l3 * e7))
            Ct = np.where(test, dd.fma(c1, l1, dd.fma(c2, l2, c0)),
                          ((2 * em - e8 * l2) - l1 * (e3 - dt2 * em)) / (l3 * e9))
        inf = l1 == -np.inf
        self.At = np.where(inf, 0.0, At)
        self.Bt = np.where(inf, 0.0, Bt)
        self.Ct = np.where(inf, 0.0, Ct)

    def step(self, u, rhs):
        """ETD.jl:229-247: ETD1 at call 1, ETD2 at call 2, ETD3 afterwards."""
        self.iteration += 1
        c = self.c
        dt = self.dt
        with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
            if self.iteration == 1:                   # ETD1stand2ndO.jl:12-26
                cdt = c * dt
                cdt2 = cdt * dt
                c2dt3 = cdt2 * cdt
                c3dt4 = c2dt3 * cdt
                test = -cdt <= 1e-4
                phi = np.where(test, dt + 0.5 * cdt2 + c2dt3 / 6 + c3dt4 / 24, dd.expm1(cdt) / c)
                phi = np.where(c == -np.inf, 0.0, phi)
                unew = dd.exp(cdt) * u + phi * rhs
            elif self.iteration == 2:                 # ETD1stand2ndO.jl:37-66
                dt2 = self.dt2
                cp2 = c * c
                cdt = c * dt
                cdtp2 = cdt * dt
                c2dtp3 = cdtp2 * cdt
                c3dtp4 = c2dtp3 * cdt
                em = dd.expm1(cdt)
                c2dt2 = c * c * dt2
                dtp2 = dt * dt
                dtp3 = dtp2 * dt
                dtp4 = dtp3 * dt
                test = -cdt <= 1e-4
                At = np.where(test,
                              dt + cdtp2 / 2 + c2dtp3 / 6 + c3dtp4 / 24 + dtp2 / (2 * dt2)
                              + (c * dtp3) / (6 * dt2) + (cp2 * dtp4) / (24 * dt2),
                              (em - c * (dt - dt2 * em)) / c2dt2)
                Bt = np.where(test, (-(dtp2 / (2 * dt2)) - (c * dtp3) / (6 * dt2) - (cp2 * dtp4) / (24 * dt2)),
                              (cdt - em) / c2dt2)
                inf = c == -np.inf
                At = np.where(inf, 0.0, At)
                Bt = np.where(inf, 0.0, Bt)
                unew = dd.exp(cdt) * u + (At * rhs + Bt * self.fm1)
            else:
                if self.adaptive:                     # set_coefficients!, ETD.jl:116-123
                    self.set_ABCt()
                unew = self.At * rhs + (self.Bt * self.fm1 + (self.Ct * self.fm2 + dd.exp(c * dt) * u))
        self.fm2 = self.fm1
        self.fm1 = rhs.copy()
        return unew


# ----------------------------------------------------------------------------------
# The simulation — src/models.jl, src/FluidFlowSimulation.jl
# ----------------------------------------------------------------------------------

STATS_HEADER = ("iteration,time,u1,u2,u3,u1p2,u2p2,u3p2,kh,kv,kaniso,k,dissh,dissv,diss,"
                "nlh,nlv,pressh,pressv,tnlh,tnlv,tdiss")


PLANE_KINDS = ("rfForcing", "cRfForcing", "nRfForcing", "cNRfForcing", "aForcing", "QfForcing")


class PlaneForcing:
    """The reference's forcing of the kz = 0 plane (forcing.jl:6-114 rfForcing,
    cforcing.jl:1-97 cRfForcing, nrforcing.jl nRfForcing, cnrforcing.jl cNRfForcing,
    aforcing.jl aForcing, qfforcing.jl:1-81 QfForcing): horizontal velocity of the kx-ky
    modes in 2D shells |k_h| <= kf (aForcing: mode by mode), scaled per shell, plus a few
    (0, 0, kz) modes that take 1 % of the power; applied after the integrator
    (add_Rf_forcing!, forcing_types.jl:54-64)."""

    def __init__(self, p: "Params", g: Grid, lfilter: bool = False):
        self.p, self.g = p, g
        # compute_shells2D (utils.jl:161-182) over the stored half plane, all ky
        self.nsh = min(g.nxh, g.ny // 2)
        self.maxdk = max(g.kx[1], g.ky[1])
        kh = np.zeros(self.nsh)
        cnt = np.zeros(self.nsh, dtype=np.int64)
        for j in range(g.ny):
            for i in range(g.nxh):
                K = math.sqrt(g.kx[i] ** 2 + g.ky[j] ** 2)
                ii = int(np.rint(K / self.maxdk))
                if ii >= self.nsh:
                    break
                kh[ii] += K
                cnt[ii] += 1
        self.kh = kh / cnt
        kf = p.pf_kf
        if p.plane_forcing == "QfForcing":
            # build_Qf_power_spectrum! (forcing_types.jl:303-330)
            R = np.zeros(self.nsh)
            integral = 0.0
            for i in range(1, self.nsh):
                if self.kh[i] <= kf:
                    term = math.exp(-((self.kh[i] - p.pf_qkf) / p.pf_qc) ** 2)
                    R[i] = p.pf_qp * term
                    integral += term
            R /= integral
            if lfilter:
                d2 = p.filter_width ** 2
                for i in range(1, self.nsh):
                    if self.kh[i] <= kf:
                        G = math.exp((-d2 / 24) * (self.kh[i] * self.kh[i]))
                        R[i] *= G * G
            self.R = R
        elif p.plane_forcing == "aForcing":
            # per-mode state over the kz = 0 plane (aforcing.jl); Zf by calculate_Zf(d,kf,kx,ky)
            Kz = np.sqrt(g.kx[None, :] ** 2 + (g.ky ** 2)[:, None])
            if p.pf_zf_tanh:
                self.Zf2 = np.tanh((kf - Kz) / (0.25 * kf)) * np.where((kf - Kz) <= 0.0, 0.0, 1.0)
            else:
                self.Zf2 = (Kz <= kf).astype(np.float64)
            shape = (g.ny, g.nxh)
            self.R2, self.Em2, self.factor2 = np.zeros(shape), np.zeros(shape), np.zeros(shape)
        else:
            if p.pf_zf_tanh:   # calculate_Zf (utils.jl:184-198)
                self.Zf = np.array([math.tanh((kf - k) / (0.25 * kf)) * (0.0 if (kf - k) <= 0.0 else 1.0)
                                    for k in self.kh])
            else:
                self.Zf = (self.kh <= kf).astype(np.float64)
            self.R = np.zeros(self.nsh)
            self.Ef = np.zeros(self.nsh)      # the shell energy of the last call (Eh.N files)
            self.Em = np.zeros(self.nsh)
            self.factor = np.zeros(self.nsh)
            self.N = np.zeros(self.nsh)
            self.Nm1 = np.zeros(self.nsh)
        # plane modes: shell index n (0-based) of each (ky, kx) with the force loop's
        # K = sqrt(muladd(kx, kx, ky^2))
        K = np.sqrt(dd.fma(*np.broadcast_arrays(g.kx[None, :], g.kx[None, :], (g.ky ** 2)[:, None])))
        self.nmode = np.rint(K / self.maxdk).astype(np.int64)
        Ks = np.sqrt(g.kx[None, :] ** 2 + (g.ky ** 2)[:, None])
        self.nspec = np.rint(Ks / self.maxdk).astype(np.int64)
        self.cf = np.where(np.arange(g.nxh) > 0, 2.0, 1.0)[None, :]
        self.Kmode = K
        self.keep = g.keep[0]
        self.hp = self.vp = 0.0

    def plane_spectrum(self, u, mag: bool):
        """calculate_u1u2_spectrum! / calculate_u1u2_mag_spectrum! (spectrum.jl:1-65) on kz = 0."""
        a2 = np.abs(u[0][0]) ** 2 + np.abs(u[1][0]) ** 2
        v = self.cf * np.sqrt(a2) if mag else 0.5 * self.cf * a2
        E = np.zeros(self.nsh)
        ok = self.keep & (self.nspec < self.nsh)
        np.add.at(E, self.nspec[ok], v[ok])
        return E

    def nn_spectrum(self, u, rhs):
        """calculate_nn_spectrum! (nrforcing.jl / cnrforcing.jl:103-126): per shell,
        cf (proj(u1, rhs1 - nu k^2 u1) + proj(u2, rhs2 - nu k^2 u2)) on kz = 0."""
        g, nu = self.g, self.p.nu
        k2 = g.kx[None, :] ** 2 + (g.ky ** 2)[:, None]
        u1, u2, r1, r2 = u[0][0], u[1][0], rhs[0][0], rhs[1][0]
        v = self.cf * (_proj(u1, r1 - (nu * k2) * u1) + _proj(u2, r2 - (nu * k2) * u2))
        N = np.zeros(self.nsh)
        ok = self.keep & (self.nspec < self.nsh)
        np.add.at(N, self.nspec[ok], v[ok])
        return N

    def initialize(self, u, rhs=None):
        """initialize! of the forcing (forcing_types.jl:66-73,107-119, aforcing.jl): the
        target spectrum of the initial field (no targSpectrum.dat); nRf/cNRf also N = Nm1
        from the initial right-hand side; aForcing its per-mode energies."""
        kind = self.p.plane_forcing
        if kind == "aForcing":
            self.Em2 = 0.5 * self.cf * (np.abs(u[0][0]) ** 2 + np.abs(u[1][0]) ** 2)
        elif kind != "QfForcing":
            self.Em = self.plane_spectrum(u, False)
            if kind in ("nRfForcing", "cNRfForcing"):
                self.N = self.nn_spectrum(u, rhs)
                self.Nm1 = self.N.copy()

    def __call__(self, u, dt, it, cfl, variable_dt, rhs=None, dt2=None):
        """The force (fx, fy) for this step and hp, vp."""
        p, g = self.p, self.g
        kf = p.pf_kf
        nz = g.nz
        fx = np.zeros_like(u[0])
        fy = np.zeros_like(u[1])
        if p.plane_forcing == "aForcing":
            return self._a_forcing(u, dt, fx, fy)
        sel = self.keep & (self.nmode >= 1) & (self.nmode < self.nsh)
        sel &= np.where(self.nmode < self.nsh, self.kh[np.minimum(self.nmode, self.nsh - 1)] <= kf, False)
        u1, u2 = u[0][0], u[1][0]
        vk = list(range(1, 6)) + [nz - k for k in range(1, 6)]   # Julia k = 2..6 and NZ-k+2
        if p.plane_forcing == "QfForcing":
            Ef = self.plane_spectrum(u, True)
            umag = np.sqrt(np.abs(u1) ** 2 + np.abs(u2) ** 2)
            n = np.minimum(self.nmode, self.nsh - 1)
            fkn = dt * self.R[n] * 0.99 / Ef[n]
            with np.errstate(divide="ignore", invalid="ignore"):
                s1 = np.where(sel, (u1 / umag) * fkn, 0.0)
                s2 = np.where(sel, (u2 / umag) * fkn, 0.0)
            fx[0], fy[0] = s1, s2
            fv = np.sum(self.cf * (_proj(u1, s1 / dt) + _proj(u2, s2 / dt)))
            hp = fv
            usq = sum(abs(u[0][k, 0, 0]) ** 2 + abs(u[1][k, 0, 0]) ** 2 for k in (3, 4, 5, nz - 3, nz - 4, nz - 5))
            f = dt * hp * (1 - 0.99) / (usq * 0.99)
            vp = 0.0
            for k in (3, 4, 5, nz - 3, nz - 4, nz - 5):
                fx[k, 0, 0] = u[0][k, 0, 0] * f
                fy[k, 0, 0] = u[1][k, 0, 0] * f
                vp += _proj(u[0][k, 0, 0], fx[k, 0, 0] / dt) + _proj(u[1][k, 0, 0], fy[k, 0, 0] / dt)
        else:
            kind = p.plane_forcing
            if kind in ("rfForcing", "nRfForcing"):
                ts = dt / cfl
                if variable_dt and it <= 3:
                    ts /= (0.1, 0.2, 0.4, 0.8)[it]
                omega = 2 * math.pi / (p.pf_tf * ts)
            elif kind == "cRfForcing":                         # ts = Tf, omega = 2 pi / ts
                omega = 2 * math.pi / p.pf_tf
            else:                                              # cNRfForcing: ts = Tf, omega = 2 pi / (Tf ts)
                omega = 2 * math.pi / (p.pf_tf * p.pf_tf)
            Ef = self.plane_spectrum(u, False)
            self.Ef = Ef
            alpha = p.pf_alpha
            eps = np.finfo(np.float64).eps
            nl = kind in ("nRfForcing", "cNRfForcing")
            if nl:                                             # nrforcing.jl: copyto!(Nm1, N); N = nn spectrum
                self.Nm1 = self.N.copy()
                self.N = self.nn_spectrum(u, rhs)
            for i in range(1, self.nsh):
                if self.kh[i] <= kf:
                    if nl:
                        self.R[i] += dt * (-2 * alpha * omega * (self.R[i] + self.N[i])
                                           - (self.N[i] - self.Nm1[i]) / dt2 - omega * omega * (Ef[i] - self.Em[i]))
                    else:
                        self.R[i] += dt * (-2 * alpha * omega * self.R[i] - omega * omega * (Ef[i] - self.Em[i]))
                    self.R[i] = max(0.0, self.R[i])
                    self.factor[i] = math.sqrt(self.R[i] / max(Ef[i], eps)) * self.Zf[i] * dt
            fac = self.factor[np.minimum(self.nmode, self.nsh - 1)]
            s1 = np.where(sel, u1 * fac, 0.0)
            s2 = np.where(sel, u2 * fac, 0.0)
            fx[0], fy[0] = s1, s2
            ff = np.sum(self.cf * (np.abs(s1) ** 2 + np.abs(s2) ** 2))
            fv = np.sum(self.cf * (_proj(u1, s1) + _proj(u2, s2)))
            hp = ff * 0.5 / dt + fv / dt
            umag = sum(math.sqrt(abs(u[0][k, 0, 0]) ** 2 + abs(u[1][k, 0, 0]) ** 2) for k in vk)
            f = dt * math.sqrt(2.0 * hp * (1.0 - 0.99)) / umag
            ff = fv = 0.0
            for k in vk:
                fx[k, 0, 0] = u[0][k, 0, 0] * f
                fy[k, 0, 0] = u[1][k, 0, 0] * f
                ff += abs(fx[k, 0, 0]) ** 2 + abs(fy[k, 0, 0]) ** 2
                fv += _proj(u[0][k, 0, 0], fx[k, 0, 0]) + _proj(u[1][k, 0, 0], fy[k, 0, 0])
            vp = ff * 0.5 / dt + fv / dt
        self.hp, self.vp = float(hp), float(vp)
        return fx, fy

    def _vertical(self, u, fx, fy, dt, hp):
        """(0, 0, kz) modes, kz = +-1..+-5: 1 % of the horizontal power (forcing.jl:86-113)."""
        nz = self.g.nz
        vk = list(range(1, 6)) + [nz - k for k in range(1, 6)]
        umag = sum(math.sqrt(abs(u[0][k, 0, 0]) ** 2 + abs(u[1][k, 0, 0]) ** 2) for k in vk)
        f = dt * math.sqrt(2.0 * hp * (1.0 - 0.99)) / umag
        ff = fv = 0.0
        for k in vk:
            fx[k, 0, 0] = u[0][k, 0, 0] * f
            fy[k, 0, 0] = u[1][k, 0, 0] * f
            ff += abs(fx[k, 0, 0]) ** 2 + abs(fy[k, 0, 0]) ** 2
            fv += _proj(u[0][k, 0, 0], fx[k, 0, 0]) + _proj(u[1][k, 0, 0], fy[k, 0, 0])
        return ff * 0.5 / dt + fv / dt

    def _a_forcing(self, u, dt, fx, fy):
        """aForcing (aforcing.jl): the ODE per kz = 0 mode with 0 < |k_h| <= kf, ts = 10 dt."""
        p = self.p
        omega = 2 * math.pi / (p.pf_tf * (10 * dt))
        alpha, eps = p.pf_alpha, np.finfo(np.float64).eps
        sel = self.keep & (self.Kmode > 0) & (self.Kmode <= p.pf_kf)
        u1, u2 = u[0][0], u[1][0]
        Ef = 0.5 * self.cf * (np.abs(u1) ** 2 + np.abs(u2) ** 2)
        R = self.R2 + dt * (-2 * alpha * omega * self.R2 - omega * omega * (Ef - self.Em2))
        R = np.maximum(0.0, R)
        self.R2 = np.where(sel, R, self.R2)
        with np.errstate(divide="ignore", invalid="ignore"):
            fac = np.sqrt(self.R2 / np.maximum(Ef, eps)) * self.Zf2 * dt
        self.factor2 = np.where(sel, fac, self.factor2)
        s1 = np.where(sel, u1 * self.factor2, 0.0)
        s2 = np.where(sel, u2 * self.factor2, 0.0)
        fx[0], fy[0] = s1, s2
        ff = np.sum(self.cf * (np.abs(s1) ** 2 + np.abs(s2) ** 2))
        fv = np.sum(self.cf * (_proj(u1, s1) + _proj(u2, s2)))
        hp = ff * 0.5 / dt + fv / dt
        self.hp, self.vp = float(hp), float(self._vertical(u, fx, fy, dt, hp))
        return fx, fy


def stats_header(p: Params) -> str:
    """``statsheader`` (stats.jl:1-7); plug-in order = sim_fields (macros.jl:48)."""
    cols = [STATS_HEADER]
    if p.scalar:
        cols.append("scalar,scalarp2,dscalardxp2,dscalardyp2,dscalardzp2,scalardiss")
    if p.density:
        cols.append("rho,rhop2,drhodxp2,drhodyp2,drhodzp2,rhodiss,trhodiss,bflux" + (",rhopr" if p.rho_les else "")
                    + (",rhohdiss" if p.rho_hv else ""))
    if p.les:
        cols.append("prh,prv,praniso,pr")
    if p.plane_forcing == "aForcing":
        cols.append("hp,vp")                                     # statsheader(a::AForcing)
    elif p.forcing or p.plane_forcing:
        cols.append("hp,vp,tp")
    if p.hv:
        cols.append("hdissh,hdissv,hdiss")
    return ",".join(cols)


def barrier_f(k, i, p):
    """log(esp(|k|, i, p, 1/4)) of the spectral barrier (hyperviscosity_types.jl:40-48)."""
    a = np.abs(k)
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        e = np.where(a <= i, 1.0, np.where(a < p, np.exp(-((a - i) * (a - i)) / (p ** 0.25 - a ** 0.25)), 0.0))
        return np.log(e)


def barrier_c(g, k2, mnu, i, p):
    """muladd(k2, -nu, f(|k|)) on the retained modes, 0 elsewhere (init_c_spectral_barrier!
    fills only XRANGE x YRANGE x ZRANGE, ETD.jl:71-82)."""
    f = np.where(g.keep, barrier_f(np.sqrt(k2), i, p), 0.0)
    with np.errstate(invalid="ignore"):
        c = dd.fma(k2, np.full_like(k2, mnu), np.where(np.isinf(f), 0.0, f))
    # f = log(0) = -inf (beyond endk, or exp underflow) makes muladd -inf: the ETD coefficients
    # are then 0 and the mode is removed (ETD.jl:182-191)
    return np.where(g.keep, np.where(np.isinf(f), -np.inf, c), 0.0)


def barrier_w(k2, i, p):
    """The barrier as a stats/spectrum weight: -inf counts 0 (stats.jl:1160-1161)."""
    f = barrier_f(np.sqrt(k2), i, p)
    return np.where(np.isinf(f), 0.0, f)


def _proj(a, b):
    """``proj(a,b)`` (forcing.jl:4): Re(a) Re(b) + Im(a) Im(b)."""
    return a.real * b.real + a.imag * b.imag


def scales_numbers_from(u1p2, u2p2, u3p2, k, tdiss, L, D, nu, density, n2):
    """The scalar part of ``stats`` (stats.jl:64-165) given the integral lengths
    L = (L11..L33), the derivative means D = (du1dy2, du1dx2, du2dy2, du2dx2), the
    viscosity and, with density, N^2 = g_z * drho/dz (calculate_N,
    density_stratification_types.jl:32-34). Returns (Scales.txt row, Numbers.txt row)
    without iteration and time."""
    L11, L12, L13, L21, L22, L23, L31, L32, L33 = L
    du1dyp2, du1dxp2, du2dyp2, du2dxp2 = D
    u1p2, u2p2, u3p2, k, tdiss = (np.float64(x) for x in (u1p2, u2p2, u3p2, k, tdiss))
    with np.errstate(divide="ignore", invalid="ignore"):
        uh = np.sqrt((u1p2 + u2p2) / 2)
        urms = np.sqrt((u1p2 + u2p2 + u3p2) / 3)
        lam12 = np.sqrt(2 * u1p2 / du1dyp2)
        lam21 = np.sqrt(2 * u2p2 / du2dxp2)
        Lhh = (L11 + L22) / 2
        Thh = Lhh / urms
        laml = np.sqrt(2 * (u1p2 + u2p2) / (du1dxp2 + du2dyp2))
        lamt = np.sqrt(2 * (u1p2 + u2p2) / (du1dyp2 + du2dxp2))
        Lhv = (L13 + L23) / 2
        Lvv = L33
        Lvh = (L31 + L32) / 2
        Lt = np.sqrt(k * k * k) / tdiss
        Tt = k / tdiss
        Lk = np.sqrt(np.sqrt(nu * nu * nu / tdiss))
        Tk = np.sqrt(nu / tdiss)
        lamg = np.sqrt(15 * nu / tdiss) * urms
        lensv = [Lk, Lt, lamg, laml, lamt, Lhh, Lvv, Lhv, Lvh, lam12, lam21, L11, L12, L13, L21, L22, L23, L31,
                 L32, L33]
        Reh = uh * Lhh / nu
        Reh1 = (Lhh / Lk) ** (4 / 3)
        Relg = urms * lamg / nu
        Relg1 = (lamg / Lk) ** (4 / 3)
        Rell = urms * laml / nu
        Rell1 = (laml / Lk) ** (4 / 3)
        Relt = urms * lamt / nu
        Relt1 = (lamt / Lk) ** (4 / 3)
        if density:
            Nb = np.sqrt(n2)
            Lb = 2 * np.pi * urms / Nb
            Lo = np.sqrt(tdiss / (Nb * Nb * Nb))
            Lom = np.sqrt(tdiss / (Nb * Nb * Nb / (8 * np.pi * np.pi * np.pi)))
            Tb = 2 * np.pi / Nb
            Tbm = 1 / Nb
            Reb = (Lo / Lk) ** (4 / 3)
            Rebm = (Lom / Lk) ** (4 / 3)
            Frh = 2 * np.pi * uh / (Nb * Lhh)
            Frh1 = Lhv / Lhh
            lens = lensv + [Lb, Lo, Lom, Tk, Tt, Thh, Tb, Tbm]
            anums = [Reh, Reh1, Relg, Rell, Relt, Relg1, Rell1, Relt1, Reb, Rebm, Frh, Frh1]
        else:
            lens = lensv + [Tk, Tt, Thh]
            anums = [Reh, Reh1, Rell, Relt, Rell1, Relt1]
    return [float(x) for x in lens], [float(x) for x in anums]


def _sym33(Sr):
    """3x3 symmetric tensor field from the 5 traceless components xx, xy, xz, yy, yz."""
    xx, xy, xz, yy, yz = Sr
    zz = -xx - yy
    return np.array([[xx, xy, xz], [xy, yy, yz], [xz, yz, zz]])


def _antisym(v):
    """AntiSymTen(v) of FluidTensors, taken as the cross-product matrix [v]x (A b = v x b),
    so that AntiSymTen(w/2) is the rotation tensor (grad u - grad u^T)/2 for w = curl u."""
    x, y, z = v
    o = np.zeros_like(x)
    return np.array([[o, -z, y], [z, o, -x], [-y, x, o]])


def _mm(a, b):
    return np.einsum("ik...,kj...->ij...", a, b)


def _ddot(a, b):
    return np.einsum("ij...,ij...->...", a, b)


def _to5(t):
    """Traceless symmetric tensor field -> the 5 stored components."""
    return np.stack([t[0, 0], t[0, 1], t[0, 2], t[1, 1], t[1, 2]])


def les_stress(p: "Params", Sr, wr):
    """tau of the pointwise LES models in physical space (calc_les!, les_real_calc.jl:13-139),
    and the model's eddy viscosity nu_t (the density / scalar eddy diffusivity, :116-134):
    Smagorinsky nu_t = c^2 D^2 |S| (:77-79); Vreman (:132-139, VremanLESModel.jl); the
    production-viscosity model (ProductionViscosityLESModel.jl); Silvis (silvismodel.jl);
    the stable non-linear model (stablenonlinearmodel.jl); the SandP P term
    cb D^2 Lie(S, AntiSymTen(w/2)) (:104-111). |S| is the Frobenius norm sqrt(S:S);
    Lie(A, B) = A B - B A."""
    S = _sym33(Sr)
    d2 = p.filter_width ** 2
    c = p.smag_c
    ss = _ddot(S, S)
    m = p.les_model
    with np.errstate(divide="ignore", invalid="ignore"):
        if m == "Smagorinsky":
            xx, xy, xz, yy, yz = Sr
            zz = -xx - yy
            nrm = np.sqrt(xx * xx + yy * yy + zz * zz + 2.0 * (xy * xy + xz * xz + yz * yz))
            nut = c * c * d2 * nrm
            t = 2.0 * nut * S
        elif m == "Vreman":
            a = S + _antisym(-0.5 * wr)
            b = d2 * _mm(np.swapaxes(a, 0, 1), a)
            B = b[0, 0] * (b[1, 1] + b[2, 2]) + b[1, 1] * b[2, 2] - (b[0, 1] ** 2 + b[0, 2] ** 2 + b[1, 2] ** 2)
            B = np.where(B < 0.0, 0.0, B)
            nut = c * np.sqrt(B / _ddot(a, a))
            t = 2.0 * nut * S
        elif m == "productionViscosity":
            W = _antisym(-0.5 * wr)
            q = c * d2 * (_ddot(_mm(W, W), S) - _ddot(_mm(S, S), S)) / (2 * ss)
            nut = np.where(ss == 0.0, 0.0, np.maximum(0.0, q))
            t = 2.0 * nut * S
        elif m == "Silvis":
            Sw = np.einsum("ij...,j...->i...", S, wr)
            fv = np.sqrt(_ddot(Sw[:, None], Sw[:, None])) / (np.sqrt(ss) * np.sqrt(np.sum(wr * wr, axis=0)))
            nut = c * c * d2 * fv * fv * fv * np.sqrt(ss) / 2
            nup = p.les_cp * d2 * fv * fv * fv * fv / 4
            Om = _antisym(0.5 * wr)
            t = 2.0 * nut * S + nup * (_mm(S, Om) - _mm(Om, S))
        elif m == "stableNonLinear":
            W = _antisym(-0.5 * wr)
            T = _mm(W, W) - (_mm(S, W) - _mm(W, S)) - _mm(S, S)
            T = T - (np.trace(T) / 3.0) * np.eye(3).reshape(3, 3, *([1] * (T.ndim - 2)))
            q = c * d2 * (_ddot(_mm(W, W), S) - _ddot(_mm(S, S), S)) / (2 * ss)
            mnu = np.where(ss == 0.0, 0.0, -np.minimum(0.0, q))
            nut = np.where(ss == 0.0, 0.0, np.maximum(0.0, q))      # stable_nl_eddy_viscosity's nu
            t = c * d2 * T + 2.0 * mnu * S
        else:
            raise ValueError(m)
        if p.sandp_cb:
            Om = _antisym(0.5 * wr)
            t = t + (p.sandp_cb * d2) * (_mm(S, Om) - _mm(Om, S))
    return _to5(t), nut


class OracleSimulation:
    """FP64 restatement of the reference Simulation for the in-scope plug-ins."""

    def __init__(self, p: Params, u_phys, rho_phys=None):
        self.p = p
        g = self.g = Grid(p.nx, p.ny, p.nz, p.lx, p.ly, p.lz, p.cutoff)
        self.iteration = p.start
        self.time = p.start_time
        self.u = np.stack([np.asarray(x, dtype=np.float64) for x in u_phys])   # physical at first
        self.rho = None                   # density, or the passive scalar phi
        if p.fld:
            self.rho = (np.zeros((p.nz, p.ny, p.nx)) if rho_phys is None
                        else np.asarray(rho_phys, dtype=np.float64))
        # c = -nu k^2 (init_c!, ETD.jl:60-69) or muladd(k2, -nu, k2^M * -nuh) (init_c_hv!,
        # ETD.jl:84-95), with k2 = muladd(KX,KX, muladd(KY,KY, KZ*KZ))
        k2 = dd.fma(*np.broadcast_arrays(g.KX, g.KX, dd.fma(*np.broadcast_arrays(g.KY, g.KY, g.KZ * g.KZ))))
        c = k2 * (-p.nu)
        if p.hv and p.hv_kind == "barrier":               # init_c_spectral_barrier! (ETD.jl:71-82)
            if p.ab3:
                raise ValueError("spectralBarrier has no AB3 form in the reference")
            c = barrier_c(g, k2, -p.nu, p.hv_initk, p.hv_endk)
        elif p.hv:
            km = k2.copy()
            for _ in range(p.hv_m - 1):
                km = km * k2
            c = dd.fma(k2, np.full_like(k2, -p.nu), km * (-p.hv_nu))
        self.k2_ref = k2
        if p.integrator == "Euller":
            self.ts = Euler(p.variable_dt, p.dt)
        elif p.ab3:
            self.ts = AB3(p.variable_dt, p.dt)
        else:
            self.ts = ETD3(p.variable_dt, p.dt, c)
        if p.fld:
            alpha = p.nu / (p.density_pr if p.density else p.scalar_pr)
            if p.integrator == "Euller":
                self.rts = Euler(p.variable_dt, p.dt)
            elif p.ab3:
                self.rts = AB3(p.variable_dt, p.dt)
            elif p.scalar and p.hv and p.hv_kind == "barrier":
                self.rts = ETD3(p.variable_dt, p.dt, barrier_c(g, k2, -alpha, p.hv_initk, p.hv_endk))
            elif p.scalar and p.hv:
                # the scalar's ETD3rdO takes the velocity's hyperviscosity (simulationtypes.jl
                # :336 passes the hyperviscositytype of :293-305): muladd(k2, -alpha, k2^M -nuh)
                self.rts = ETD3(p.variable_dt, p.dt, dd.fma(k2, np.full_like(k2, -alpha), km * (-p.hv_nu)))
            elif p.rho_hv == "barrier":                   # the density's own (density_stratification_types.jl:137-176)
                self.rts = ETD3(p.variable_dt, p.dt, barrier_c(g, k2, -alpha, p.rho_hv_initk, p.rho_hv_endk))
            elif p.rho_hv == "power":
                kr = k2.copy()
                for _ in range(p.rho_hv_m - 1):
                    kr = kr * k2
                self.rts = ETD3(p.variable_dt, p.dt, dd.fma(k2, np.full_like(k2, -alpha), kr * (-p.rho_hv_nu)))
            else:
                self.rts = ETD3(p.variable_dt, p.dt, k2 * (-alpha))
            self.alpha = alpha
        self.gvec = np.zeros(3)
        if p.density:
            self.gvec[p.gravity_dir] = p.gravity
        # reference reductionh[1] / density reduction[1] with Julia threads = 1
        self.slot_u = 0.0
        self.slot_rho = 0.0
        self.nlstats = (1.0, 1.0)
        self.pressstats = (1.0, 1.0)
        self.nlstats_fil = (1.0, 1.0)                      # simulationtypes.jl:94-95
        self.stats_rows = []
        self.stats_fil_rows = []                           # Stats_fil.txt (stats.jl:48-52)
        # STAT_FIL weight Gaussfilter(SPEC_FIL_D2, k.k)^2 (utils.jl:220-225, stats.jl)
        if p.spec_fil:
            G = np.exp((-p.fil_d2 / 24) * g.K2)
            self.G2 = G * G
            mx = int(np.argmax(g.dealias[0, 0, :])) if g.dealias[0, 0, :].any() else g.nxh
            self.ix_last = mx - 1                          # last index of XRANGE
        else:
            self.G2 = None
        self.scales_rows = []
        self.numbers_rows = []
        self.spectra = {}
        self.force = None
        self.hp = self.vp = 0.0
        self.pforce = PlaneForcing(p, g, lfilter=p.les) if p.plane_forcing else None
        self.pforce_xy = None
        self.umax_hist = []
        # Optional Delta t sequence that replaces the CFL value of each set_dt! call, in
        # call order (parity tests feed the engine's own sequence here); newdt_hist
        # records the values set_dt! produced or took.
        self.dt_sequence = None
        self.newdt_hist = []
        # piomelliSmagorinsky's coefficient state (c, cm1, dtm1)
        self.piom_c = self.piom_cm1 = None
        self.piom_dtm1 = 0.0
        self.piom_cp = self.piom_cpm1 = None
        self.piom_dtpm1 = 0.0

    # ---------------------------------------------------------------- time helpers
    def get_dt(self):
        return self.ts.dt

    def is_stats_time(self):
        return self.iteration % self.p.dt_stat == 0

    def is_spec_time(self):
        return self.iteration % self.p.dt_spec == 0

    # ---------------------------------------------------------------- initialize!
    def initialize(self):
        """``initialize!(s)`` (FluidFlowSimulation.jl:67-91)."""
        g = self.g
        self.u = g.myfourier(self.u)
        if self.p.fld:
            self.rho = g.myfourier(self.rho)
        self.calculate_rhs()
        dt_now = self.get_dt()
        if self.pforce is not None:                               # initialize!(s.forcing, s)
            self.pforce.initialize(self.u, self.rhs)
        self.ts.initialize(self.rhs, dt_now)
        if self.p.fld:
            self.rts.initialize(self.rhorhs, dt_now)

    # ---------------------------------------------------------------- calculate_rhs!
    def calculate_rhs(self):
        """``calculate_rhs!`` (models.jl:19-51)."""
        p, g = self.p, self.g
        u = self.u
        KX, KY, KZ = g.KX, g.KY, g.KZ
        stats_t = self.is_stats_time()
        spec_t = self.is_spec_time()
        # fourierspacep1! (models.jl:63-119): w = (i k) x u ; S = symouter(i k, u)
        ikx, iky, ikz = 1j * KX, 1j * KY, 1j * KZ
        w = np.stack([iky * u[2] - ikz * u[1], ikz * u[0] - ikx * u[2], ikx * u[1] - iky * u[0]])
        if p.les:
            S = np.stack([ikx * u[0], 0.5 * (ikx * u[1] + iky * u[0]), 0.5 * (ikx * u[2] + ikz * u[0]),
                          iky * u[1], 0.5 * (iky * u[2] + ikz * u[1])])
        # realspace! (models.jl:121-214)
        ur = g.real(u)
        wr = g.real(w)
        kspec = None
        if spec_t or stats_t:                                     # :130-134
            kspec = g.myfourier(0.5 * (ur[0] * ur[0] + ur[1] * ur[1] + ur[2] * ur[2]))
        if p.fld:
            rhor = g.real(self.rho)
        if p.les:
            Sr = g.real(S)
            if p.les_model in ("dynamicSmagorinsky", "piomelliSmagorinsky"):
                taur, nut = self.dynamic_smagorinsky(u, ur, S, Sr, w, wr)
            else:
                taur, nut = les_stress(p, Sr, wr)
        # realspacecalculation! (models.jl:236-280): rhs = u x w ; flux = -rho u
        nl = np.stack([ur[1] * wr[2] - ur[2] * wr[1], ur[2] * wr[0] - ur[0] * wr[2],
                       ur[0] * wr[1] - ur[1] * wr[0]])
        if p.fld:
            flux = -rhor[None] * ur                               # models.jl:265-275
            if p.rho_les:
                # calc_les! (les_real_calc.jl:116-134): nu_t grad rho (+ (c D^2 / 2) w x grad rho),
                # grad rho = real!(i k rho) (fourierspacep1!, models.jl:110-115)
                gr = g.real(np.stack([ikx * self.rho, iky * self.rho, ikz * self.rho]))
                lf = nut[None] * gr
                if p.rho_les == "vorticity":
                    cr = p.rho_les_c * p.filter_width ** 2 / 2
                    lf = lf + cr * np.stack([wr[1] * gr[2] - wr[2] * gr[1], wr[2] * gr[0] - wr[0] * gr[2],
                                             wr[0] * gr[1] - wr[1] * gr[0]])
                flux = flux + lf
        if p.les:
            # writeoutput's LES fields of this calculate_rhs! (output.jl:22-42)
            self.les_out = {n: taur[i] for i, n in enumerate(("T11", "T12", "T13", "T22", "T23"))}
            if p.les_model in ("dynamicSmagorinsky", "piomelliSmagorinsky"):
                self.les_out["cs"] = self.dyn_c
                if p.les_dynp:
                    self.les_out["cp"] = self.dyn_cp
            if p.density and p.rho_les:
                self.les_out.update(dflux1=lf[0], dflux2=lf[1], dflux3=lf[2])
        if p.variable_dt:                                         # find_max, utils.jl:247-258
            m = float(np.max(np.abs(ur)))
            self.slot_u = max(m, self.slot_u) if p.reference_cfl_slot else m
            self.umax_hist.append(m)
            if p.density:
                mr = float(np.max(np.abs(rhor)))
                self.slot_rho = max(mr, self.slot_rho) if p.reference_cfl_slot else mr
        nlh = g.myfourier(nl)
        nlh[:, 0, 0, 0] = 0.0                                     # models.jl:174
        # u round trip + projection (models.jl:192-193)
        self.u = u = g.project(g.myfourier(ur))
        if p.fld:
            fluxh = g.myfourier(flux)
            self.rho = g.myfourier(rhor)
        tauh = g.myfourier(taur) if p.les else None
        # set_dt! (time_step_functions.jl:86-129)
        if p.variable_dt:
            self.set_dt()
        if spec_t:
            sp = self.spectrum_u()
            ikflux = (1j * (KX * fluxh[0] + (KY * fluxh[1] + KZ * fluxh[2]))) if p.density else None
            sp.update(self.spectra_write_spec(nlh, kspec, tauh, ikflux))
            self.spectra[self.iteration] = sp
        if stats_t:                                               # models.jl:38-46
            if p.density and p.rho_les:   # the flux scalar_les_stats reads (stats.jl:1032-1053)
                self.ikflux_st = 1j * (KX * fluxh[0] + (KY * fluxh[1] + KZ * fluxh[2]))
            self.nlstats = self.non_linear_stats(nlh, kspec)
            self.pressstats = self.pressure_stats(nlh, kspec, tauh)
        # fourierspacep2! (models.jl:282-364)
        rhs = nlh.copy()
        if p.ab3:                                                 # explicit viscosity :320-326
            if p.hv:
                rhs = rhs + (g.K2 * (-p.nu) + (g.K2 ** p.hv_m) * (-p.hv_nu))[None] * u
            else:
                rhs = rhs + (g.K2 * (-p.nu))[None] * u
        if p.les:                                                 # :328-332
            rhs = rhs + self.div_tau(tauh)
        if p.density:                                             # :334-336
            for d in range(3):
                if self.gvec[d] != 0.0:
                    rhs[d] = rhs[d] + self.rho * self.gvec[d]
        rhs = g.project(rhs)                                      # :338-339
        rhs[:, g.dealias] = 0.0
        self.rhs = rhs
        self.kspec = kspec
        self.tauh = tauh
        if p.fld:                                                 # div!, vectorfunctions.jl:93-103
            wdir = u[p.fld_dir]
            rr = 1j * (KX * fluxh[0] + (KY * fluxh[1] + KZ * fluxh[2])) + (-p.fld_grad) * wdir
            if p.ab3:
                rr = rr + (-self.alpha * g.K2) * self.rho
            rr[g.dealias] = 0.0
            self.rhorhs = rr

    def dynamic_smagorinsky(self, u, ur, S, Sr, w=None, wr=None):
        """The dynamic Smagorinsky model (dynamic_smagorinsky.jl:3-217, les_real_calc.jl:3-11,
        71-73): test-filtered u and S (fourierspacep1!, models.jl:99-108), Sa = D^2 |S| S and
        L = u u filtered over the full spectrum (fourierspace_dynamic_les_calculation!), the
        Germano coefficient c = clamp(L:M / 2 M:M, -1, 1) with L = traceless(u^ u^ - (uu)^)
        and M = (D^^2 + D^2) |S^| S^ - (D^2 |S| S)^, c averaged by the same filter
        (average_c!, dynamic_piomelli.jl:13-26), then nu_t = max(cmin, min(0.4, c)) D^2 |S|.
        The filter is Gaussfilter (utils.jl:220-225): exp(-D^^2 k^2 / 24).

        With the dynamic P tensor (dynamicSandP / piomelliSandP, les_types.jl:199-330):
        P = D^2 Lie(S, W), W = AntiSymTen(w/2) (times the extrapolated cp for piomelliSandP,
        cp = cpm1 = 0.09 at construction), filtered like Sa; w^ = G w; P^ = Lie(S^, W^);
        dynamicSandP: cp = clamp(L:Mp / Mp:Mp, -1, 1), Mp = (D^^2 + D^2) P^ - P~;
        piomelliSandP: cp = clamp((tau^ + L):Mp / Mp:Mp, -1, 1), Mp = (D^^2 + D^2) P^, tau^ =
        P~ (+ Sa~ with piomelliSmagorinsky, whose own tau^ then includes P~ too); cp averaged
        like c; tau += clamp(cp, -0.8, 0.8) D^2 Lie(S, W) (dynamic_smagorinsky.jl:3-217,
        les_real_calc.jl:104-106)."""
        p, g = self.p, self.g
        d2 = p.filter_width ** 2
        dh2 = p.les_test_width ** 2
        G = np.exp((-dh2 / 24) * g.K2)

        def full_filter(f):            # fullfourier!, multiply by G on every mode, real!
            c = sfft.rfftn(f, axes=(-3, -2, -1), workers=_WORKERS) * (1.0 / g.N)
            return g.real(c * G)

        def nrm5(t):
            xx, xy, xz, yy, yz = t
            zz = -xx - yy
            return np.sqrt(xx * xx + yy * yy + zz * zz + 2.0 * (xy * xy + xz * xz + yz * yz))

        uf = g.real(G[None] * u)                                   # u^ (physical)
        Sh = g.real(G[None] * S)                                   # S^ (physical)
        piomelli = p.les_model == "piomelliSmagorinsky"
        dynp = p.les_dynp
        if dynp:
            def lie5(S5, wv):
                A, B = _sym33(S5), _antisym(0.5 * wv)
                return _to5(_mm(A, B) - _mm(B, A))
            lie_r = lie5(Sr, wr)
            if dynp == "piomelliSandP":     # calc_cstar! on cp (dynamic_smagorinsky.jl:22-35)
                if self.piom_cp is None:
                    self.piom_cp = np.full(ur[0].shape, 0.09)
                    self.piom_cpm1 = np.full(ur[0].shape, 0.09)
                dt = self.get_dt()
                dtf = 1.0 if dt == 0.0 else dt
                dtm1f = dtf if self.piom_dtpm1 == 0.0 else self.piom_dtpm1
                if self.iteration == 0:
                    self.piom_cpm1 = self.piom_cp.copy()
                cpstar = (dtf / dtm1f) * (self.piom_cp - self.piom_cpm1) + self.piom_cp
                self.piom_cpm1 = self.piom_cp
                self.piom_dtpm1 = dt
                Pa = (cpstar * d2)[None] * lie_r                   # cp D^2 Lie(S, W)
            else:
                Pa = d2 * lie_r                                    # D^2 Lie(S, W)
            Paf = np.stack([full_filter(x) for x in Pa])
            wh = g.real(G[None] * w)                               # w^ (physical)
        if piomelli:
            # calc_cstar! (dynamic_smagorinsky.jl:9-19, dynamic_piomelli.jl:1-11): the last
            # averaged coefficient extrapolated in time, c* = c + (dt/dtm1)(c - cm1); c and
            # cm1 start at 0.0289 (les_types.jl:261-266), cm1 := c at iteration 0
            if self.piom_c is None:
                self.piom_c = np.full(ur[0].shape, 0.0289)
                self.piom_cm1 = np.full(ur[0].shape, 0.0289)
            dt = self.get_dt()
            dtf = 1.0 if dt == 0.0 else dt
            dtm1f = dtf if self.piom_dtm1 == 0.0 else self.piom_dtm1
            if self.iteration == 0:
                self.piom_cm1 = self.piom_c.copy()
            r = dtf / dtm1f
            cstar = r * (self.piom_c - self.piom_cm1) + self.piom_c
            self.piom_cm1 = self.piom_c
            self.piom_dtm1 = dt
            Sa = (2 * cstar * d2 * nrm5(Sr))[None] * Sr            # 2 c* D^2 |S| S
        else:
            Sa = d2 * nrm5(Sr)[None] * Sr                          # D^2 |S| S
        ux, uy, uz = ur
        Lr = np.stack([ux * ux, ux * uy, ux * uz, uy * uy, uy * uz, uz * uz])
        Saf = np.stack([full_filter(x) for x in Sa])
        Lf = np.stack([full_filter(x) for x in Lr])
        a, b, c_ = uf
        L6 = np.stack([a * a, a * b, a * c_, b * b, b * c_, c_ * c_]) - Lf
        tr = (L6[0] + L6[3] + L6[5]) / 3
        L6[0] -= tr
        L6[3] -= tr
        L6[5] -= tr
        def ddot_n(t5, M5):           # (t + L) : M / (M:M), t traceless (5 components)
            mxx, mxy, mxz, myy, myz = M5
            mzz = -mxx - myy
            mm = mxx * mxx + myy * myy + mzz * mzz + 2.0 * (mxy * mxy + mxz * mxz + myz * myz)
            nxx, nxy, nxz, nyy, nyz, nzz = mxx / mm, mxy / mm, mxz / mm, myy / mm, myz / mm, mzz / mm
            txx, txy, txz, tyy, tyz = t5
            tzz = -txx - tyy
            return ((txx + L6[0]) * nxx + (tyy + L6[3]) * nyy + (tzz + L6[5]) * nzz
                    + 2.0 * ((txy + L6[1]) * nxy + (txz + L6[2]) * nxz + (tyz + L6[4]) * nyz))

        if piomelli:
            # c = (tau^ + L) : M / (M:M), M = 2 (D^^2 + D^2) |S^| S^ (dynamic_smagorinsky.jl:174-185)
            M5 = (2 * (dh2 + d2) * nrm5(Sh))[None] * Sh
            mxx, mxy, mxz, myy, myz = M5
            mzz = -mxx - myy
            mm = mxx * mxx + myy * myy + mzz * mzz + 2.0 * (mxy * mxy + mxz * mxz + myz * myz)
            nxx, nxy, nxz, nyy, nyz, nzz = mxx / mm, mxy / mm, mxz / mm, myy / mm, myz / mm, mzz / mm
            txx, txy, txz, tyy, tyz = Saf + Paf if dynp == "piomelliSandP" else Saf
            tzz = -txx - tyy
            cv = ((txx + L6[0]) * nxx + (tyy + L6[3]) * nyy + (tzz + L6[5]) * nzz
                  + 2.0 * ((txy + L6[1]) * nxy + (txz + L6[2]) * nxz + (tyz + L6[4]) * nyz))
            cf = np.maximum(-1.0, np.minimum(1.0, cv))
        else:
            M5 = (dh2 + d2) * nrm5(Sh)[None] * Sh - Saf
            mxx, mxy, mxz, myy, myz = M5
            mzz = -mxx - myy
            lm = (L6[0] * mxx + L6[3] * myy + L6[5] * mzz + 2.0 * (L6[1] * mxy + L6[2] * mxz + L6[4] * myz))
            mm = mxx * mxx + myy * myy + mzz * mzz + 2.0 * (mxy * mxy + mxz * mxz + myz * myz)
            cf = np.maximum(-1.0, np.minimum(1.0, 0.5 * (lm / mm)))
        cf = full_filter(cf)                                       # average_c!
        if piomelli:
            self.piom_c = cf
        cpf = None
        if dynp:
            Ph = lie5(Sh, wh)                                      # Lie(S^, AntiSymTen(w^/2))
            dsum = dh2 + d2
            if dynp == "dynamicSandP":
                Mp = dsum * Ph - Paf
                mxx, mxy, mxz, myy, myz = Mp
                mzz = -mxx - myy
                lm = (L6[0] * mxx + L6[3] * myy + L6[5] * mzz + 2.0 * (L6[1] * mxy + L6[2] * mxz + L6[4] * myz))
                mm = mxx * mxx + myy * myy + mzz * mzz + 2.0 * (mxy * mxy + mxz * mxz + myz * myz)
                cpv = lm / mm
            else:
                cpv = ddot_n(Saf + Paf if piomelli else Paf, dsum * Ph)
            cpf = full_filter(np.maximum(-1.0, np.minimum(1.0, cpv)))   # average_c! of cp
            if dynp == "piomelliSandP":
                self.piom_cp = cpf
        self.dyn_c, self.dyn_cp = cf, cpf
        nut = np.maximum(p.les_cmin, np.minimum(0.4, cf)) * d2 * nrm5(Sr)
        tau = 2.0 * nut[None] * Sr
        if p.sandp_cb:                # SandP: tau += cb D^2 Lie(S, W) (les_real_calc.jl:98-104)
            A, B = _sym33(Sr), _antisym(0.5 * wr)
            tau = tau + (p.sandp_cb * d2) * _to5(_mm(A, B) - _mm(B, A))
        if dynp:
            tau = tau + (np.maximum(-0.8, np.minimum(0.8, cpf)) * d2)[None] * lie_r
        return tau, nut

    def div_tau(self, tauh):
        """(i k) . tau for a symmetric traceless tau (models.jl:330)."""
        g = self.g
        xx, xy, xz, yy, yz = tauh
        zz = -xx - yy
        ikx, iky, ikz = 1j * g.KX, 1j * g.KY, 1j * g.KZ
        return np.stack([ikx * xx + iky * xy + ikz * xz,
                         ikx * xy + iky * yy + ikz * yz,
                         ikx * xz + iky * yz + ikz * zz])

    # ---------------------------------------------------------------- set_dt!
    def set_dt(self):
        """``set_dt!(s)`` (time_step_functions.jl:86-129)."""
        p, g = self.p, self.g
        umax = self.slot_u
        dx = 2 * math.pi * p.ly / p.ny
        cfl = p.cfl
        it = self.iteration
        if it == 0:
            cfl *= 0.1
        elif it == 1:
            cfl *= 0.2
        elif it == 2:
            cfl *= 0.4
        elif it == 3:
            cfl *= 0.8
        with np.errstate(divide="ignore"):
            newdt = cfl * dx / umax if umax != 0 else math.inf
        if p.density:
            rmax = self.slot_rho
            gn = abs(p.gravity)
            den = rmax * gn
            cap = cfl * math.sqrt(dx / den) if den > 0 else math.inf
            newdt = min(newdt, cap)
        if it > 3:
            dt = self.get_dt()
            if newdt < dt:
                newdt = max(dt / 1.25, newdt)
            else:
                newdt = min(1.25 * dt, newdt)
        if self.dt_sequence is not None:
            newdt = float(self.dt_sequence[len(self.newdt_hist)])
        self.newdt_hist.append(newdt)
        self.ts.set_dt(newdt)
        if p.fld:   # density and passive scalar integrators (time_step_functions.jl:126-128)
            self.rts.set_dt(newdt)

    # ---------------------------------------------------------------- forcing (new)
    def compute_forcing(self):
        """Isotropic band forcing at constant power (no reference counterpart).

        E_f = sum_{0<|k|<=kf} 1/2 w |u|^2 ; f = dt * eps/(2 E_f) * u on that band,
        applied after the integrator like the reference's add_forcing! hook
        (forcing_types.jl:49-64, time_step_functions.jl:72-80).
        """
        p, g = self.p, self.g
        u = self.u
        band = (g.K2 <= p.forcing_kf ** 2) & (g.K2 > 0) & g.keep
        w = g.w
        e = 0.5 * w * (np.abs(u[0]) ** 2 + np.abs(u[1]) ** 2 + np.abs(u[2]) ** 2)
        Ef = float(np.sum(e[band]))
        coef = p.forcing_power / (2.0 * Ef) if Ef > 0 else 0.0
        dt = self.get_dt()
        f = np.where(band[None], (dt * coef) * u, 0.0)
        self.force = f
        wb = np.broadcast_to(w, band.shape)
        sh = _proj(u[0], f[0]) + _proj(u[1], f[1]) + 0.5 * (np.abs(f[0]) ** 2 + np.abs(f[1]) ** 2)
        sv = _proj(u[2], f[2]) + 0.5 * np.abs(f[2]) ** 2
        self.hp = float(np.sum((wb * sh)[band])) / dt
        self.vp = float(np.sum((wb * sv)[band])) / dt

    # ---------------------------------------------------------------- advance_in_time!
    def plane_force(self):
        """s.forcing(s) of the kz = 0 plane family, from the current u (models.jl:6-9)."""
        p = self.p
        self.pforce_xy = self.pforce(self.u, self.get_dt(), self.iteration, p.cfl, p.variable_dt, self.rhs,
                                     self.ts.dt2)
        self.hp, self.vp = self.pforce.hp, self.pforce.vp

    def advance(self):
        """``advance_in_time!`` (models.jl:3-17)."""
        p, g = self.p, self.g
        self.calculate_rhs()
        if p.forcing:
            self.compute_forcing()
        if self.pforce is not None:
            self.plane_force()
            if self.is_spec_time():     # write_spec_forcing (spec.jl:148-170, 262-271)
                fx, fy = self.pforce_xy
                v = (_proj(self.u[0], fx) + _proj(self.u[1], fy)) / self.get_dt()
                H, V = self.calculate_specHV(v)
                self.spectra[self.iteration]["forcing_h.specH"] = H
                self.spectra[self.iteration]["forcing_h.specV"] = V
        if self.is_stats_time():
            self.write_stats()
        # time_step! (models.jl:468-472) -> VectorTimeStep (time_step_functions.jl:72-80)
        if p.ab3:
            u = self.ts.step(self.u, self.rhs)
        else:
            u = self.ts.step(self.u, self.rhs)
        if p.forcing:
            u = u + self.force
        if self.pforce is not None:                               # add_Rf_forcing!, forcing_types.jl:54-64
            u = u.copy()
            u[0] = u[0] + self.pforce_xy[0]
            u[1] = u[1] + self.pforce_xy[1]
        self.u = g.project(u)
        self.u[:, g.dealias] = 0.0
        if p.fld:
            self.rho = self.rts.step(self.rho, self.rhorhs)
            self.rho[g.dealias] = 0.0
        self.iteration += 1
        self.time += self.get_dt()

    def run(self, nsteps):
        for _ in range(nsteps):
            self.advance()

    def finalize(self):
        """Tail of ``run_simulation`` (FluidFlowSimulation.jl:46-49)."""
        self.calculate_rhs()
        if self.p.forcing:
            self.compute_forcing()
        if self.pforce is not None:
            self.plane_force()
        self.write_stats()

    # ---------------------------------------------------------------- stats
    def _wsum(self, a):
        return float(np.sum(self.g.w * a))

    def non_linear_stats(self, nl, ke):
        """stats.jl:897-917 (with STAT_FIL also the G^2-weighted sums, :919-949, kept in
        nlstats_fil)."""
        g = self.g
        u = self.u
        r = [nl[0] - 1j * g.KX * ke, nl[1] - 1j * g.KY * ke, nl[2] - 1j * g.KZ * ke]
        hh = _proj(r[0], u[0]) + _proj(r[1], u[1])
        vv = _proj(r[2], u[2])
        h = self._wsum(hh)
        v = self._wsum(vv)
        if self.G2 is not None:
            self.nlstats_fil = (self._wsum(hh * self.G2), self._wsum(vv * self.G2))
        if self.p.variable_dt and self.p.reference_cfl_slot:
            self.slot_u = h
        return h, v

    def pressure_stats(self, nl, ke, tauh):
        """stats.jl:750-814."""
        p, g = self.p, self.g
        u = self.u
        r = np.stack([nl[0] - 1j * ke * g.KX, nl[1] - 1j * ke * g.KY, nl[2] - 1j * ke * g.KZ])
        if p.les:
            r = r + self.div_tau(tauh)
        if p.density:
            for d in range(3):
                if self.gvec[d] != 0.0:
                    r[d] = r[d] + self.rho * self.gvec[d]
        kd = g.KX * r[0] + g.KY * r[1] + g.KZ * r[2]
        with np.errstate(divide="ignore", invalid="ignore"):
            p1 = -kd / g.K2
        p1[0, 0, 0] = 0.0
        hh = _proj(u[0], p1 * g.KX) + _proj(u[1], p1 * g.KY)
        vv = _proj(u[2], p1 * g.KZ)
        if self.G2 is not None:
            # STAT_FIL branch (stats.jl:832-893): the G^2-weighted terms are added to the
            # unfiltered sums (eeh += leeh*G2) and the filtered sums stay 0
            hh = hh + hh * self.G2
            vv = vv + vv * self.G2
        h = self._wsum(hh)
        v = self._wsum(vv)
        if self.p.variable_dt and self.p.reference_cfl_slot:
            self.slot_u = h
        return h, v

    def velocity_row(self):
        """``velocity_stats`` + ``stats`` (stats.jl:64-219), Stats.txt column order."""
        p, g = self.p, self.g
        u = self.u
        a2 = [np.abs(u[i]) ** 2 for i in range(3)]
        u12, u22, u32 = (self._wsum(a) for a in a2)
        kh = (u12 + u22) / 2
        kv = u32 / 2
        k = kh + kv
        kaniso = 2 * kv / kh
        eh_raw = self._wsum(g.K2 * (a2[0] + a2[1]))
        ev_raw = self._wsum(g.K2 * a2[2])
        eh, ev = p.nu * eh_raw, p.nu * ev_raw
        nlh, nlv = self.nlstats
        ph, pv = self.pressstats
        row = [u[0][0, 0, 0].real, u[1][0, 0, 0].real, u[2][0, 0, 0].real, u12, u22, u32,
               kh, kv, kaniso, k, eh, ev, eh + ev, nlh, nlv, ph, pv, -(nlh + ph), (nlv + pv)]
        tdiss = eh + ev
        extra = []
        slot = None
        # derivative variances used for the Taylor scales (stats.jl:79-94); the last one
        # (dx_squared_mean of u2) is what stays in reductionh[1]
        slot = self._wsum(g.KX ** 2 * a2[1])
        if p.scalar:                                              # scalar_stats, stats.jl:221-233
            phi = self.rho
            r2 = np.abs(phi) ** 2
            d1 = self._wsum(g.KX ** 2 * r2)
            d2 = self._wsum(g.KY ** 2 * r2)
            d3 = self._wsum(g.KZ ** 2 * r2)
            extra += [phi[0, 0, 0].real, self._wsum(r2), d1, d2, d3, self.alpha * (d1 + d2 + d3)]
        if p.density:
            rho = self.rho
            r2 = np.abs(rho) ** 2
            rho2 = self._wsum(r2)
            d1 = self._wsum(g.KX ** 2 * r2)
            d2 = self._wsum(g.KY ** 2 * r2)
            d3 = self._wsum(g.KZ ** 2 * r2)
            rhodiss = self.alpha * (d1 + d2 + d3)
            bf_raw = self._wsum(_proj(u[p.gravity_dir], rho))
            bflux = -self.gvec[p.gravity_dir] * bf_raw
            # density_stratification_types.jl:46-87: trhodiss = rhodiss (+ rhopr) (+ rhohdiss);
            # each sum leaves its raw total in the density's reduction slot
            trd, tail, rslot = rhodiss, [], bf_raw
            if p.rho_les:   # scalar_les_stats (stats.jl:1032-1053): rhopr = -sum proj(i k.flux, rho)
                pr_raw = self._wsum(_proj(self.ikflux_st, rho))
                trd += -pr_raw
                tail.append(-pr_raw)
                rslot = pr_raw
            if p.rho_hv:   # scalar_hvis_stats (stats.jl:1086-1110, 1145-1171), trhodiss += it
                rh_raw = self._wsum(self._rho_hv_weight() * r2)
                rh = -rh_raw if p.rho_hv == "barrier" else p.rho_hv_nu * rh_raw
                trd += rh
                tail.append(rh)
                rslot = rh_raw
            extra += [rho[0, 0, 0].real, rho2, d1, d2, d3, rhodiss, trd, bflux] + tail
            if p.variable_dt and p.reference_cfl_slot:
                self.slot_rho = rslot
        if p.les:
            t = self.div_tau(self.tauh)
            hraw = self._wsum(_proj(t[0], u[0]) + _proj(t[1], u[1]))
            vraw = self._wsum(_proj(t[2], u[2]))
            prh, prv = -hraw, -vraw
            extra += [prh, prv, (2 * prv) / prh, prh + prv]
            tdiss += prh + prv
            slot = hraw
        if p.plane_forcing == "aForcing":
            extra += [self.hp, self.vp]
        elif p.forcing or p.plane_forcing:
            extra += [self.hp, self.vp, self.hp + self.vp]
        if p.hv:
            hw = self._hv_weight()
            hraw = self._wsum(hw * (a2[0] + a2[1]))
            vraw = self._wsum(hw * a2[2])
            sc = -1.0 if p.hv_kind == "barrier" else p.hv_nu   # spectral_barrier_stats: -sums
            extra += [sc * hraw, sc * vraw, sc * (hraw + vraw)]
            tdiss += sc * (hraw + vraw)
            slot = hraw
        if self.G2 is not None:
            fil, fslot = self._velocity_row_fil(a2)
            self.fil_row = fil
            if fslot is not None and not (p.les or p.hv):
                slot = fslot
        if p.variable_dt and p.reference_cfl_slot:
            self.slot_u = slot
        return row + [tdiss] + extra

    def _hv_weight(self):
        """Per-mode weight of the velocity hyperviscosity stats: (k^2)^M or the barrier."""
        p, g = self.p, self.g
        if p.hv_kind == "barrier":
            return barrier_w(g.K2, p.hv_initk, p.hv_endk)
        return g.K2 ** p.hv_m

    def _rho_hv_weight(self):
        p, g = self.p, self.g
        if p.rho_hv == "barrier":
            return barrier_w(g.K2, p.rho_hv_initk, p.rho_hv_endk)
        return g.K2 ** p.rho_hv_m

    def _velocity_row_fil(self, a2):
        """The Stats_fil.txt row (STAT_FIL branches of velocity_stats, scalar_stats,
        buoyancy_flux, les_stats, hyperviscosity_stats; stats.jl:168-233, 354-376,
        501-524, 563-606, 637-677, 707-747, density_stratification_types.jl:46-87,
        192-210): every quadratic sum weighted by G^2, the means unweighted, the pressure
        columns 0 (their filtered sums are never accumulated, stats.jl:880-891), and the
        forcing columns as in Stats.txt. dx_squared_mean's filtered sum keeps only the
        last kx of each line (`ee_fil = ...` where the others accumulate, stats.jl:370).
        Returns the row and the value the reductionh slot holds after the scalar and
        density stats (None without them)."""
        p, g = self.p, self.g
        u, G2 = self.u, self.G2
        ws = lambda a: self._wsum(a * G2)   # noqa: E731
        u12, u22, u32 = (ws(a) for a in a2)
        kh = (u12 + u22) / 2
        kv = u32 / 2
        k = kh + kv
        eh, ev = p.nu * ws(g.K2 * (a2[0] + a2[1])), p.nu * ws(g.K2 * a2[2])
        nlh, nlv = self.nlstats_fil
        ph = pv = 0.0
        row = [u[0][0, 0, 0].real, u[1][0, 0, 0].real, u[2][0, 0, 0].real, u12, u22, u32,
               kh, kv, 2 * kv / kh, k, eh, ev, eh + ev, nlh, nlv, ph, pv, -(nlh + ph), (nlv + pv)]
        tdiss = eh + ev
        extra = []
        fslot = None

        def scalar_fil(f):
            r2 = np.abs(f) ** 2
            i = self.ix_last
            d1 = float(np.sum((g.w * g.KX ** 2 * r2 * G2)[:, :, i]))
            d2, d3 = ws(g.KY ** 2 * r2), ws(g.KZ ** 2 * r2)
            return [f[0, 0, 0].real, ws(r2), d1, d2, d3, self.alpha * (d1 + d2 + d3)], d3

        if p.scalar:
            vals, fslot = scalar_fil(self.rho)
            extra += vals
        if p.density:
            vals, fslot = scalar_fil(self.rho)
            bf_raw = ws(_proj(u[p.gravity_dir], self.rho))
            trd, tail, fslot = vals[-1], [], bf_raw
            if p.rho_les:   # the filtered sum goes through reductionh (density_stratification_types.jl:58)
                pr_raw = ws(_proj(self.ikflux_st, self.rho))
                trd += -pr_raw
                tail.append(-pr_raw)
                fslot = pr_raw
            if p.rho_hv:
                rh_raw = ws(self._rho_hv_weight() * np.abs(self.rho) ** 2)
                rh = -rh_raw if p.rho_hv == "barrier" else p.rho_hv_nu * rh_raw
                trd += rh
                tail.append(rh)
                fslot = rh_raw
            extra += vals + [trd, -self.gvec[p.gravity_dir] * bf_raw] + tail
        if p.les:
            t = self.div_tau(self.tauh)
            prh = -ws(_proj(t[0], u[0]) + _proj(t[1], u[1]))
            prv = -ws(_proj(t[2], u[2]))
            extra += [prh, prv, (2 * prv) / prh, prh + prv]
            tdiss += prh + prv
        if p.plane_forcing == "aForcing":
            extra += [self.hp, self.vp]
        elif p.forcing or p.plane_forcing:
            extra += [self.hp, self.vp, self.hp + self.vp]
        if p.hv:
            hw = self._hv_weight()
            hraw = ws(hw * (a2[0] + a2[1]))
            vraw = ws(hw * a2[2])
            sc = -1.0 if p.hv_kind == "barrier" else p.hv_nu
            extra += [sc * hraw, sc * vraw, sc * (hraw + vraw)]
            tdiss += sc * (hraw + vraw)
        return row + [tdiss] + extra, fslot

    def write_stats(self):
        """``writestats`` (stats.jl:39-62): one row each of Stats.txt, Scales.txt, Numbers.txt."""
        row = self.velocity_row()
        lens, anums = self.scales_numbers(row)
        head = [float(self.iteration), float(self.time)]
        self.stats_rows.append(head + row)
        if self.G2 is not None:
            self.stats_fil_rows.append(head + self.fil_row)
        self.scales_rows.append(head + lens)
        self.numbers_rows.append(head + anums)

    def scales_numbers(self, row):
        """Length/time scales and dimensionless numbers of ``stats`` (stats.jl:64-165) from
        the spectral state: integral lengths (integral_lenght_x/y/z, stats.jl:952-980) and
        the derivative means dx/dy_squared_mean (stats.jl:334-400)."""
        p, g = self.p, self.g
        u = self.u
        a2 = [np.abs(u[i]) ** 2 for i in range(3)]
        u1p2, u2p2, u3p2 = row[3], row[4], row[5]
        k, tdiss = row[9], row[19]
        uh = np.sqrt((u1p2 + u2p2) / 2)
        urms = np.sqrt((u1p2 + u2p2 + u3p2) / 3)
        w = np.where(np.arange(g.nxh) > 0, 2.0, 1.0)[None, None, :]
        kx0 = (g.kx == 0)[None, None, :]
        ky0 = (g.ky == 0)[None, :, None]
        kz0 = (g.kz == 0)[:, None, None]
        keep = g.keep

        def il(a, up2):
            up2 = np.float64(up2)
            rx = np.sum(np.where(keep & kx0, a, 0.0))
            ry = np.sum(np.where(keep & ky0, w * a, 0.0))
            rz = np.sum(np.where(keep & kz0, w * a, 0.0))
            with np.errstate(divide="ignore", invalid="ignore"):
                return p.lx * rx * np.pi / up2, p.ly * ry * np.pi / up2, p.lz * rz * np.pi / up2

        L11, L12, L13 = il(a2[0], u1p2)
        L21, L22, L23 = il(a2[1], u2p2)
        L31, L32, L33 = il(a2[2], u3p2)
        d1dy = self._wsum(g.KY ** 2 * a2[0])
        d1dx = self._wsum(g.KX ** 2 * a2[0])
        d2dy = self._wsum(g.KY ** 2 * a2[1])
        d2dx = self._wsum(g.KX ** 2 * a2[1])
        return scales_numbers_from(u1p2, u2p2, u3p2, k, tdiss, (L11, L12, L13, L21, L22, L23, L31, L32, L33),
                                   (d1dy, d1dx, d2dy, d2dx), p.nu, p.density,
                                   self.gvec[2] * p.density_gradient if p.density else 0.0)

    # ---------------------------------------------------------------- spectra
    def spectrum_u(self):
        """``spectrum_u`` + ``calculate_specHV`` (spec.jl:316-327, 424-450).

        Returns dict with the horizontal/vertical parts binned into H and V spectra:
        keys 'u_h.specH', 'u_h.specV', 'u.specH', 'u_v.specH', 'u_v.specV'.
        """
        u = self.u
        hout = 0.5 * (_proj(u[0], u[0]) + _proj(u[1], u[1]))
        vout = 0.5 * _proj(u[2], u[2])
        hH, hV = self.calculate_specHV(hout)
        vH, vV = self.calculate_specHV(vout)
        out = {"u_h.specH": hH, "u_h.specV": hV, "u.specH": hH + vH, "u_v.specH": vH, "u_v.specV": vV}
        if self.G2 is not None:                     # u_fil: filter_spectrum! (spec.jl:17-20, 452-472)
            hH, hV = self.calculate_specHV(self.G2 * hout)
            vH, vV = self.calculate_specHV(self.G2 * vout)
            out.update({"u_fil_h.specH": hH, "u_fil_h.specV": hV, "u_fil.specH": hH + vH,
                        "u_fil_v.specH": vH, "u_fil_v.specV": vV})
        return out

    def spectra_write_spec(self, nl, ke, tauh, ikflux):
        """The other spectra of ``write_spec`` (spec.jl:1-146, 196-422), binned by
        ``calculate_specHV``: viscous, non-linear, pressure, LES, hyperviscous and the
        density spectra (buoyancy_v, rho, rhodiss, rhonl). Keys '<field>.specH/V'."""
        p, g = self.p, self.g
        u = self.u
        out = {}
        G2 = self.G2

        def put(name, field, fil=None):
            H, V = self.calculate_specHV(field)
            out[name + ".specH"], out[name + ".specV"] = H, V
            if G2 is not None and fil is not None:   # the filter_spectrum! twin (spec.jl:13-142)
                H, V = self.calculate_specHV(G2 * field)
                out[fil + ".specH"], out[fil + ".specV"] = H, V

        k2 = g.KX * g.KX + (g.KY * g.KY + g.KZ * g.KZ)
        uh_ = 0.5 * (_proj(u[0], u[0]) + _proj(u[1], u[1]))
        uv_ = 0.5 * _proj(u[2], u[2])
        put("vis_h", 2 * p.nu * k2 * uh_, "vis_fil_h")            # spectrum_viscosity
        put("vis_v", 2 * p.nu * k2 * uv_, "vis_fil_v")
        r = np.stack([nl[0] - 1j * g.KX * ke, nl[1] - 1j * g.KY * ke, nl[2] - 1j * g.KZ * ke])
        put("nl_h", _proj(r[0], u[0]) + _proj(r[1], u[1]), "nl_fil_h")   # spectrum_non_linear
        put("nl_v", _proj(r[2], u[2]), "nl_fil_v")
        if p.les:
            dt_ = self.div_tau(tauh)
            r = r + dt_
        if p.density:
            for d in range(3):
                if self.gvec[d] != 0.0:
                    r[d] = r[d] + self.rho * self.gvec[d]
        kd = g.KX * r[0] + g.KY * r[1] + g.KZ * r[2]
        with np.errstate(divide="ignore", invalid="ignore"):
            p1 = -kd / g.K2
        p1[0, 0, 0] = 0.0
        put("press_h", _proj(u[0], p1 * g.KX) + _proj(u[1], p1 * g.KY), "press_fil_h")   # spectrum_pressure
        put("press_v", _proj(u[2], p1 * g.KZ), "press_fil_v")
        if p.les:
            put("les_h", _proj(dt_[0], u[0]) + _proj(dt_[1], u[1]))       # spectrum_les
            put("les_v", _proj(dt_[2], u[2]))
        if p.hv:   # spectrum_hyperviscosity / spectrum_spectral_barrier (spec.jl:273-314)
            km = barrier_w(k2, p.hv_initk, p.hv_endk) if p.hv_kind == "barrier" else p.hv_nu * k2 ** p.hv_m
            put("hvis_h", km * (_proj(u[0], u[0]) + _proj(u[1], u[1])), "hvis_fil_h")
            put("hvis_v", km * _proj(u[2], u[2]), "hvis_fil_v")
        if p.density:
            rho = self.rho
            put("buoyancy_v", self.gvec[2] * _proj(u[2], rho), "buoyancy_fil_v")   # spectrum_buoyancy
            r2 = _proj(rho, rho)
            put("rho", r2, "rho_fil")                                     # spectrum_rho
            put("rhodiss", self.alpha * k2 * r2)                          # spectrum_rhodiss
            put("rhonl", _proj(ikflux, rho), "rhonl_fil")                 # spectrum_rhonl
            if G2 is not None:
                # rhodiss_fil: spectrum_rhodiss of the filtered rho spectrum, filtered once
                # more (spec.jl:97-108), so G^4
                H, V = self.calculate_specHV(G2 * (self.alpha * k2 * (G2 * r2)))
                out["rhodiss_fil.specH"], out["rhodiss_fil.specV"] = H, V
        return out

    def calculate_specHV(self, out):
        """spec.jl:424-450 (kx = 0 plane without the dk factors, as in the reference)."""
        g = self.g
        h = np.zeros(len(g.KH))
        v = np.zeros(len(g.KRZ))
        nk = np.rint(np.abs(g.kz) / g.DKZ).astype(np.int64)
        nj = np.rint(np.abs(g.ky) / g.MAXDKH).astype(np.int64)
        nx = np.rint(np.abs(g.kx) / g.MAXDKH).astype(np.int64)
        keep = g.keep
        o = np.where(keep, out, 0.0)
        # Bins past the end are dropped: the reference writes them under @inbounds (out of
        # bounds when ny > nx or nz differs), the engine skips them.
        def add(a, idx, val):
            ok = idx < len(a)
            np.add.at(a, idx[ok], val[ok])
        # i = 1 (kx = 0) terms
        e0 = o[:, :, 0]
        h[0] += 0.5 * float(np.sum(e0[:, nj < len(h)]))
        add(h, nj, 0.5 * np.sum(e0, axis=0))
        add(v, nk, np.sum(e0, axis=1))
        # i >= 2 terms
        e = 2.0 * o[:, :, 1:]
        add(h, nx[1:], 0.5 * g.MAXDKH * np.sum(e, axis=(0, 1)))
        add(h, nj, 0.5 * g.MAXDKH * np.sum(e, axis=(0, 2)))
        add(v, nk, g.DKZ * np.sum(e, axis=(1, 2)))
        return h, v

    # ---------------------------------------------------------------- accessors
    def u_physical(self):
        return self.g.real(self.u)

    def rho_physical(self):
        return self.g.real(self.rho)


# ----------------------------------------------------------------------------------
# Small helpers used by the known-answer tests
# ----------------------------------------------------------------------------------

def taylor_green(n: int):
    """README.md:12-20: u1 = cos x sin y sin z, u2 = -sin x cos y sin z, u3 = 0."""
    x = 2 * np.pi * np.arange(n) / n
    X = x[None, None, :]
    Y = x[None, :, None]
    Z = x[:, None, None]
    u1 = np.cos(X) * np.sin(Y) * np.sin(Z)
    u2 = -np.sin(X) * np.cos(Y) * np.sin(Z)
    u3 = np.zeros((n, n, n))
    return u1, u2, u3
