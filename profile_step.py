"""Minimal driver for profilers: set_fields + initialize + K steps of the forced-DNS workload
(or, with the fourth argument ``les``, of the stratified Smagorinsky LES workload; with
``hv``, of the large-DNS workload: hyperviscosity 1e-12 k^4, nu = 2e-4, band forcing, AB3,
the spectral initial-condition generator with k0 = 8 and modes |k_i| <= 48, the setup of
the 1024^3 configuration at any n).

    python profile_step.py [n] [FP32|FP64] [steps] [dns|les|hv]

Runs the same workload as bench.py (seeded random-phase field, k0 = 4, band forcing,
AB3 with adaptive dt, stats every 100 steps) with the default launch shapes (the
autotuner's usual picks on GB300; tuning under a profiler would time the candidates
serialised and cold) and nothing else, so a profiler's launch list is short:
k_phys_fwd_x x2, k_fwd_y, k_fwd_z_store (set_fields), one initialize! step, then
`steps` steps.
"""
import math
import sys
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parent))

import __graft_entry__ as ge  # noqa: E402


def main():
    n = int(sys.argv[1]) if len(sys.argv) > 1 else 256
    prec = sys.argv[2] if len(sys.argv) > 2 else "FP32"
    steps = int(sys.argv[3]) if len(sys.argv) > 3 else 3
    pkg = ge.load_package()
    kind = sys.argv[4] if len(sys.argv) > 4 else "dns"
    les = kind == "les"
    if kind == "hv":
        d = {"nx": str(n), "ny": str(n), "nz": str(n), "xDomainSize": "1.0", "yDomainSize": "1.0",
             "zDomainSize": "1.0", "kinematicViscosity": "2e-4", "dtStat": "100", "dtSpec": "1000000000",
             "writeTime": "1000000000", "velocityTimeStep": "Adams_Bashforth3rdO", "variableTimestepFlag": "true",
             "cfl": "0.5", "dt": "0.0001", "forcing": "isotropicBand", "forcingPower": "0.1", "forcingKf": "2.5",
             "hyperViscosity": "true", "hyperViscosityCoefficient": "1e-12", "hyperViscosityM": "2"}
        from importlib import import_module
        f = import_module(pkg.__name__ + ".fields")
        sim = pkg.Simulation.from_global(d, precision=prec)
        kc = min(48, n // 3 - 1)
        box = f.random_spectrum_modes(n, 8.0, 4001, kc)
        for c in range(3):
            sim.set_spectral(c, f.embed_half_spectrum(box[c], n, kc))
        sim.initialize()
        sim.advance_in_time(steps)
        print("ok", n, prec, sim.iteration)
        return
    if les:   # stably stratified Smagorinsky LES with density, ETD3 (the 128^3 LES configuration)
        d = {"nx": str(n), "ny": str(n), "nz": str(n), "xDomainSize": "1.0", "yDomainSize": "1.0",
             "zDomainSize": "1.0", "kinematicViscosity": "5e-4", "dtStat": "50", "dtSpec": "50",
             "writeTime": "1000000000", "velocityTimeStep": "ETD3rdO", "variableTimestepFlag": "true",
             "cfl": "0.18", "dt": "0.001", "lesModel": "Smagorinsky", "smagorinskyConstant": "0.17",
             "filterWidth": repr(2 * math.pi / n), "densityStratification": "true", "zAcceleration": "1",
             "referenceDensity": "1", "densityGradient": "1", "Pr": "1"}
        u = pkg.random_spectrum(n, k0=3.0, seed=3001)
    else:
        d = {"nx": str(n), "ny": str(n), "nz": str(n), "xDomainSize": "1.0", "yDomainSize": "1.0",
             "zDomainSize": "1.0", "kinematicViscosity": "0.001", "dtStat": "100", "dtSpec": "1000000000",
             "writeTime": "1000000000", "velocityTimeStep": "Adams_Bashforth3rdO", "variableTimestepFlag": "true",
             "cfl": "0.5", "dt": "0.001", "forcing": "isotropicBand", "forcingPower": "0.1", "forcingKf": "2.5"}
        u = pkg.random_spectrum(n, k0=4.0, seed=2001)
    sim = pkg.Simulation.from_global(d, precision=prec)
    sim.set_fields(*u, rho=np.zeros_like(u[0]) if les else None)
    sim.initialize()
    sim.advance_in_time(steps)
    print("ok", n, prec, sim.iteration)


if __name__ == "__main__":
    main()
