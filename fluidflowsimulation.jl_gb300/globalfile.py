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

from ._lib import FFS_AB3, FFS_ETD3, FFS_FP32, FFS_FP64, FFSParams, load


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
    p.write_time = int(d["writeTime"])
    integ = d.get("velocityTimeStep", "ETD3rdO")
    if integ == "Adams_Bashforth3rdO":
        p.integrator = FFS_AB3
    elif integ == "ETD3rdO":
        p.integrator = FFS_ETD3
    else:
        raise ValueError(f"velocityTimeStep {integ!r} is not supported (ETD3rdO, Adams_Bashforth3rdO)")
    p.variable_dt = 1 if _bool(d.get("variableTimestepFlag", "true")) else 0
    p.cfl = float(d.get("cfl", "0.18"))
    p.dt = parse_number(d["dt"]) if "dt" in d else 0.0
    if "hyperViscosity" in d:
        if d["hyperViscosity"] == "spectralBarrier":
            raise ValueError("hyperViscosity spectralBarrier is not supported")
        p.hyperviscosity = 1
        p.hv_nu = float(d["hyperViscosityCoefficient"])
        p.hv_m = int(d.get("hyperViscosityM", "2"))
    if "lesModel" in d:
        if d["lesModel"] != "Smagorinsky":
            raise ValueError(f"lesModel {d['lesModel']!r} is not supported (Smagorinsky)")
        p.les = 1
        p.smag_c = parse_number(d.get("smagorinskyConstant", "0.17"))
        p.filter_width = parse_number(d["filterWidth"]) if "filterWidth" in d else 0.0
    if "densityStratification" in d:
        p.density = 1
        p.density_pr = parse_number(d["Pr"])
        p.density_gradient = parse_number(d["densityGradient"])
        p.gravity = parse_number(d["zAcceleration"]) / parse_number(d["referenceDensity"])
        p.gravity_dir = {"x": 0, "y": 1, "z": 2}[d.get("gravityDirection", "z")]
        if "densityLesModel" in d or "densityHyperViscosity" in d:
            raise ValueError("density LES / density hyperviscosity are not supported")
    if "passiveScalar" in d:
        raise ValueError("passiveScalar is not supported")
    if d.get("equation", "") == "NS":
        raise ValueError("equation NS (conservation form) is not supported")
    if "forcing" in d:
        if d["forcing"] != "isotropicBand":
            raise ValueError(f"forcing {d['forcing']!r} is not supported (isotropicBand)")
        p.forcing = 1
        p.forcing_power = parse_number(d.get("forcingPower", "0.1"))
        p.forcing_kf = parse_number(d.get("forcingKf", "2.5"))
    if "referenceCflSlot" in d:
        p.reference_cfl_slot = 1 if _bool(d["referenceCflSlot"]) else 0
    if "autotune" in d:   # engine key: time the candidate launch shapes at create
        p.autotune = 1 if _bool(d["autotune"]) else 0
    prec = precision or d.get("precision", "FP64")
    p.precision = FFS_FP32 if prec.upper() == "FP32" else FFS_FP64
    p.device = device
    return p
