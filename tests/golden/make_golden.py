"""Regenerate the golden fixtures: 16^3 cases run for 10 steps by the FP64 oracle.

Each case stores its `global` keys, the initial physical fields (float64 [z, y, x]), the
spectral state after 10 steps (complex128 half spectrum [comp][z, y, kx]) and the Stats
rows. The reference (Julia + FFTW) cannot run here, so these fixtures pin the oracle and
the engine against each other and against future changes, not against the reference.

    python tests/golden/make_golden.py
"""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle.ffs_oracle import Grid, OracleSimulation, Params  # noqa: E402

N = 16
STEPS = 10


def base(**kw):
    d = {"nx": str(N), "ny": str(N), "nz": str(N), "xDomainSize": "1.0", "yDomainSize": "1.0", "zDomainSize": "1.0",
         "kinematicViscosity": "0.02", "dtStat": "3", "dtSpec": "5", "writeTime": "1000",
         "velocityTimeStep": "Adams_Bashforth3rdO", "variableTimestepFlag": "false", "cfl": "0.5", "dt": "0.01"}
    d.update(kw)
    return d


CASES = {
    "ab3_fixed": base(),
    "ab3_adaptive_forced": base(variableTimestepFlag="true", forcing="isotropicBand", forcingPower="0.1",
                                forcingKf="2.5"),
    "etd_fixed_hv": base(velocityTimeStep="ETD3rdO", hyperViscosity="true", hyperViscosityCoefficient="1e-4"),
    "etd_les_density": base(velocityTimeStep="ETD3rdO", lesModel="Smagorinsky", densityStratification="true", Pr="1",
                            densityGradient="1", zAcceleration="1", referenceDensity="1"),
}


def initial_fields(seed, density):
    rng = np.random.default_rng(seed)
    g = Grid(N, N, N)
    uh = np.stack([g.myfourier(rng.standard_normal((N, N, N))) for _ in range(3)])
    uh = g.project(uh) * np.exp(-np.sqrt(g.K2) / 3)[None]
    u = g.real(uh)
    u = u / np.sqrt(np.mean(u * u))
    rho = 0.1 * g.real(g.myfourier(rng.standard_normal((N, N, N))) * np.exp(-np.sqrt(g.K2) / 3)) if density else None
    return u, rho


def main():
    out = Path(__file__).resolve().parent
    for i, (name, d) in enumerate(sorted(CASES.items())):
        density = "densityStratification" in d
        u, rho = initial_fields(100 + i, density)
        s = OracleSimulation(Params.from_global(d), u, rho)
        s.initialize()
        s.run(STEPS)
        arrays = {"u0": u, "uh": s.u, "stats": np.array(s.stats_rows), "keys": np.array(list(d.keys())),
                  "values": np.array(list(d.values()))}
        if density:
            arrays["rho0"] = rho
            arrays["rhoh"] = s.rho
        np.savez_compressed(out / f"{name}.npz", **arrays)
        print(name, s.iteration, s.time)


if __name__ == "__main__":
    main()
