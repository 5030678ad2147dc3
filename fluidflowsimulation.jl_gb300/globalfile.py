"""The reference's `global` parameter file and its mapping onto ``ffs_params``.

``readglobal`` mirrors ReadGlobal/GlobalFileHelper (not vendored in the reference): one
``key value`` pair per line, ``//`` comments, blank lines ignored. ``parameters`` follows
``parameters(d)`` (src/simulationtypes.jl:242-365) and the grid/dealias keys of
src/Globals.jl:106-183 for the keys this engine implements; unknown keys are ignored,
as the reference ignores them.
"""
from __future__ import annotations

import math
import re
from pathlib import Path

from ._lib import FFS_AB3, FFS_ETD3, FFS_EULER, FFS_FP32, FFS_FP64, LES_MODELS, FFSParams, load


def readglobal(path: str | Path = "global") -> dict[str, str]:
    d: dict[str, str] = {}
    for raw in Path(path).read_text().splitlines():
        line = raw.strip()
        if not line or line.startswith("//") or line.startswith("#"):
            continue
        parts = line.split(None, 1)
        d[parts[0]] = parts[1].strip() if len(parts) > 1 else ""
    return d


def parse_number(s: str) -> float:
    """Numeric values as the reference evaluates them (``eval(Meta.parse(...))``):
    numbers, ``Inf``, and products with ``π``/``pi`` such as ``2π`` or ``2pi/128``."""
    t = s.strip().replace("π", "pi")
    t = re.sub(r"(\d)\s*pi", r"\1*pi", t)
    if not re.fullmatch(r"[0-9eE+\-*/(). pinfI]*", t):
        raise ValueError(f"unsupported numeric expression {s!r}")
    return float(eval(t, {"__builtins__": {}}, {"pi": math.pi, "Inf": math.inf}))


def _bool(s: str) -> bool:
    return s.strip().lower() == "true"


# constant key and default of each pointwise LES model (les_types.jl:360-395)
_LES_CONST = {"Smagorinsky": ("smagorinskyConstant", 0.17), "Vreman": ("vremanConstant", 0.032),
              "productionViscosity": ("productionConstant", 0.4), "Silvis": ("silvisConstant", math.sqrt(0.17)),
              "stableNonLinear": ("nlConstant", 0.1)}


def _set_les(p: FFSParams, d: dict[str, str]) -> None:
    """lesModel (les_types.jl:360-395): Smagorinsky, Vreman, productionViscosity, Silvis,
    stableNonLinear, dynamicSmagorinsky or piomelliSmagorinsky (les_types.jl:388-397:
    filterWidth, TestFilterWidth with default twice the filter width, cmin), or SandP (the
    P tensor term on top of sLesModel = Smagorinsky, Vreman or productionViscosity). The
    dynamic P-tensor variants dynamicSandP and piomelliSandP take sLesModel =
    dynamicSmagorinsky or piomelliSmagorinsky."""
    m = d["lesModel"]
    base = m
    if m == "SandP" and d.get("sLesModel") in ("dynamicSmagorinsky", "piomelliSmagorinsky"):
        p.sandp_cb = parse_number(d.get("pConstant", "0.09"))   # SandP on a dynamic model (les_types.jl:401-416)
        m = d["sLesModel"]
    if m in ("dynamicSandP", "piomelliSandP"):          # les_types.jl:426-455
        base = d.get("sLesModel", "")
        if base not in ("dynamicSmagorinsky", "piomelliSmagorinsky"):
            raise ValueError(f"{m} with sLesModel {base!r} is not supported (dynamicSmagorinsky, piomelliSmagorinsky)")
        p.les_dynp = 1 if m == "dynamicSandP" else 2
        m = base
    if m in ("dynamicSmagorinsky", "piomelliSmagorinsky"):
        p.les = 1
        p.les_model = LES_MODELS[m]
        p.filter_width = parse_number(d["filterWidth"]) if "filterWidth" in d else 0.0
        p.les_test_width = parse_number(d["TestFilterWidth"]) if "TestFilterWidth" in d else 0.0
        p.les_cmin = float(d["cmin"]) if "cmin" in d else 0.0
        return
    if m == "SandP":
        base = d.get("sLesModel", "")
        if base not in ("Smagorinsky", "Vreman", "productionViscosity"):
            raise ValueError(f"SandP with sLesModel {base!r} is not supported (Smagorinsky, Vreman, "
                             "productionViscosity)")
        p.sandp_cb = parse_number(d.get("pConstant", "0.09"))
    if base not in _LES_CONST:
        raise ValueError(f"lesModel {m!r} is not supported (Smagorinsky, Vreman, productionViscosity, Silvis, "
                         "stableNonLinear, dynamicSmagorinsky, piomelliSmagorinsky, SandP)")
    key, dflt = _LES_CONST[base]
    if m == "SandP" and base == "productionViscosity":
        dflt = 0.1                                           # les_types.jl:402
    p.les = 1
    p.les_model = LES_MODELS[base]
    p.smag_c = parse_number(d[key]) if key in d else dflt
    if base == "Silvis":
        p.les_cp = parse_number(d.get("silvisPConstant", "5.0"))
    if "filterWidth" in d:
        p.filter_width = parse_number(d["filterWidth"])
    elif m == "SandP" and base == "Smagorinsky":             # les_types.jl:395: twice the default
        p.filter_width = 2 * (p.lx * 2 * math.pi / p.nx) / p.cutoff
    else:
        p.filter_width = 0.0                                 # the engine's default (lx 2 pi / nx) / cutoff


PLANE_FORCING = {"rfForcing": 1, "cRfForcing": 2, "QfForcing": 3, "nRfForcing": 4, "cNRfForcing": 5, "aForcing": 6}


def parameters(d: dict[str, str], precision: str | None = None, device: int = 0) -> FFSParams:
    """Build ``ffs_params`` from a `global` dict (src/simulationtypes.jl:242-365)."""
    p = FFSParams()
    load().ffs_params_default(p)
    p.nx, p.ny, p.nz = int(d["nx"]), int(d["ny"]), int(d["nz"])
    p.lx = parse_number(d["xDomainSize"])
    p.ly = parse_number(d["yDomainSize"])
    p.lz = parse_number(d["zDomainSize"])
    p.nu = parse_number(d["kinematicViscosity"])
    if "cutoff" in d:
        p.cutoff = parse_number(d["cutoff"])
    p.start = int(d.get("start", "0"))
    p.start_time = float(d.get("startTime", "0.0"))
    p.dt_stat = int(d["dtStat"])
    p.dt_spec = int(d["dtSpec"])          # the reference raises KeyError without it (:262)
    p.spec_fil = float(d["specFil"]) if "specFil" in d else 0.0   # Globals.jl:173-178
    p.write_time = int(d["writeTime"])
    integ = d.get("velocityTimeStep", "ETD3rdO")
    if integ == "Adams_Bashforth3rdO":
        p.integrator = FFS_AB3
    elif integ == "Euller":           # simulationtypes.jl:312-313, Euller.jl
        p.integrator = FFS_EULER
    elif integ == "ETD3rdO":
        p.integrator = FFS_ETD3
    else:
        raise ValueError(f"velocityTimeStep {integ!r} is not supported (ETD3rdO, Adams_Bashforth3rdO, Euller)")
    p.variable_dt = 1 if _bool(d.get("variableTimestepFlag", "true")) else 0
    p.cfl = float(d.get("cfl", "0.18"))
    p.dt = parse_number(d["dt"]) if "dt" in d else 0.0
    if d.get("hyperViscosity") == "spectralBarrier":    # simulationtypes.jl:294-297
        p.hyperviscosity = 1
        p.hv_kind = 1
        p.hv_initk = float(d["initk"]) if "initk" in d else 0.0
        p.hv_endk = float(d["endk"]) if "endk" in d else 0.0
    elif "hyperViscosity" in d:
        p.hyperviscosity = 1
        p.hv_nu = float(d["hyperViscosityCoefficient"])
        p.hv_m = int(d.get("hyperViscosityM", "2"))
    if "densityHyperViscosity" in d:                     # density_stratification_types.jl:137-148
        if d["densityHyperViscosity"] == "spectralBarrier":
            p.rho_hv = 2
            p.rho_hv_initk = float(d["densityInitk"]) if "densityInitk" in d else 0.0
            p.rho_hv_endk = float(d["densityEndk"]) if "densityEndk" in d else 0.0
        else:
            p.rho_hv = 1
            p.rho_hv_nu = float(d["densityHyperViscosityCoefficient"])
            p.rho_hv_m = int(d.get("densityHyperViscosityM", "2"))
    if "lesModel" in d:
        _set_les(p, d)
    if "densityStratification" in d:
        p.density = 1
        p.density_pr = parse_number(d["Pr"])
        p.density_gradient = parse_number(d["densityGradient"])
        p.gravity = parse_number(d["zAcceleration"]) / parse_number(d["referenceDensity"])
        p.gravity_dir = {"x": 0, "y": 1, "z": 2}[d.get("gravityDirection", "z")]
        if "densityLesModel" in d:   # density_stratification_types.jl:176-185
            if "lesModel" not in d:
                # the reference's flux then keeps a bare grad rho (calc_les! never runs)
                raise ValueError("densityLesModel needs lesModel")
            if d["densityLesModel"] == "vorticityDiffusion":
                p.rho_les = 2
                p.rho_les_c = float(d.get("densityVorticityCoefficient", "0.1"))
            else:
                p.rho_les = 1
    if "passiveScalar" in d:   # simulationtypes.jl:320-352
        if "lesModel" in d:    # the scalar's LES diffusion (simulationtypes.jl:334-346)
            if d.get("scalarLesModel") == "vorticityDiffusion":
                p.rho_les = 2
                p.rho_les_c = float(d.get("scalarVorticityCoefficient", "1.0"))
            else:
                p.rho_les = 1
        if "densityStratification" in d:
            raise ValueError("a passive scalar together with density stratification is not supported")
        p.passive_scalar = 1
        p.scalar_pr = parse_number(d["scalarPr"])
        p.scalar_gradient = parse_number(d["scalarGradient"])
        p.scalar_dir = {"x": 0, "y": 1, "z": 2}[d.get("scalarDirection", "z")]
    if d.get("equation", "") == "NS":
        raise ValueError("equation NS (conservation form) is not supported")
    if "forcing" in d:
        f = d["forcing"]
        if f == "isotropicBand":
            p.forcing = 1
            p.forcing_power = parse_number(d.get("forcingPower", "0.1"))
            p.forcing_kf = parse_number(d.get("forcingKf", "2.5"))
        elif f in PLANE_FORCING:   # forcing_model (forcing_types.jl:335-450)
            p.plane_forcing = PLANE_FORCING[f]
            p.pf_kf = float(d["kf"])
            if f == "QfForcing":
                p.pf_qp, p.pf_qc, p.pf_qkf = (float(d[k]) for k in ("alveliusP", "alveliusC", "alveliusKf"))
            else:
                p.pf_tf, p.pf_alpha = float(d["TF"]), float(d["alphac"])
                p.pf_zf_tanh = 0 if d.get("Zf", "cutoff") == "cutoff" else 1
        else:
            raise ValueError(f"forcing {f!r} is not supported (isotropicBand, rfForcing, cRfForcing, nRfForcing, "
                             "cNRfForcing, aForcing, QfForcing)")
    if "referenceCflSlot" in d:
        p.reference_cfl_slot = 1 if _bool(d["referenceCflSlot"]) else 0
    if "autotune" in d:   # engine key: time the candidate launch shapes at create
        p.autotune = 1 if _bool(d["autotune"]) else 0
    prec = precision or d.get("precision", "FP64")
    p.precision = FFS_FP32 if prec.upper() == "FP32" else FFS_FP64
    p.device = device
    return p
