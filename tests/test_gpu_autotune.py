"""The launch-shape autotuner (ffs_params.autotune): every candidate it may pick computes
the same step, so a tuned engine matches the default one to FP32 rounding (2e-6 after 5
steps) and, in FP64, the oracle to the 1e-12 parity bar. The choice is cached per shape."""
import numpy as np
import pytest

from oracle.ffs_oracle import OracleSimulation, Params

pytestmark = pytest.mark.gpu


def gdict(n, **kw):
    d = {"nx": str(n), "ny": str(n), "nz": str(n), "xDomainSize": "1.0", "yDomainSize": "1.0",
         "zDomainSize": "1.0", "kinematicViscosity": "1e-3", "dtStat": "2", "dtSpec": "1000", "writeTime": "1000",
         "velocityTimeStep": "Adams_Bashforth3rdO", "variableTimestepFlag": "true", "cfl": "0.5", "dt": "0.001",
         "forcing": "isotropicBand", "forcingPower": "0.1", "forcingKf": "2.5"}
    d.update({k: str(v) for k, v in kw.items()})
    return d


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.parametrize("n", [128, 512])
def test_tuned_engine_matches_default(gpu_pkg, n):
    d = gdict(n)
    u = gpu_pkg.random_spectrum(n, k0=4.0, seed=21)
    sims = []
    for tune in (0, 1):
        p = gpu_pkg.parameters(d, precision="FP32")
        p.autotune = tune
        s = gpu_pkg.Simulation(p)
        s.set_fields(*u)
        s.initialize()
        s.advance_in_time(5 if n < 512 else 3)
        sims.append(s)
    a, b = sims
    assert a.tuning == "" and "->" in b.tuning
    for c in range(3):
        assert rel(b.spectral(c), a.spectral(c)) <= 2e-6, (n, c, b.tuning)
    for s in sims:
        s.close()
    p = gpu_pkg.parameters(d, precision="FP32")
    p.autotune = 1
    again = gpu_pkg.Simulation(p)
    assert "(cached)" in again.tuning
    again.close()


def test_tuned_fp64_keeps_parity(gpu_pkg):
    d = gdict(64, kinematicViscosity="0.01", variableTimestepFlag="false", dt="0.005", forcing="none")
    d.pop("forcing")
    u = gpu_pkg.random_spectrum(64, k0=3.0, seed=5)
    p = gpu_pkg.parameters(d, precision="FP64")
    p.autotune = 1
    sim = gpu_pkg.Simulation(p)
    sim.set_fields(*u)
    sim.initialize()
    sim.advance_in_time(10)
    ref = OracleSimulation(Params.from_global(d), u)
    ref.initialize()
    ref.run(10)
    for c in range(3):
        assert rel(sim.spectral(c), ref.u[c]) <= 1e-12, (c, sim.tuning)
    sim.close()


@pytest.mark.parametrize("variant", [2, 3, 4])
def test_kernel_variants_match_default_512(gpu_pkg, variant):
    """Every forced y/z form at 512^3 (line pairs, one line per thread, and half tiles:
    TX/2 kx lines a CTA with the compile-time plans) computes the default step (FP32
    rounding, 3 steps)."""
    n = 512
    d = gdict(n)
    u = gpu_pkg.random_spectrum(n, k0=4.0, seed=21)
    out = []
    for kv in (0, variant):
        p = gpu_pkg.parameters(d, precision="FP32")
        p.kernel_variant = kv
        s = gpu_pkg.Simulation(p)
        s.set_fields(*u)
        s.initialize()
        s.advance_in_time(3)
        out.append([s.spectral(c) for c in range(3)])
        s.close()
    for c in range(3):
        assert rel(out[1][c], out[0][c]) <= 2e-6, (variant, c)
