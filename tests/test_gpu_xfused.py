"""The specialised FP32 kernels (register-fused x pass, compile-time-length y/z passes;
n in {64, 128, 256, 512}; kernel_variant 2 and 3 force the line-pair and the
one-line-per-thread forms of the y/z passes) against the runtime-plan kernels and
against the FP64 oracle.

Both variants compute the same products in FP32 and differ only in the order of the
FFT's floating-point operations, so fields agree to ~1e-7 relative; the bar is 2e-6
after 5 steps (fields); stats rows agree to 1e-5 relative plus 1e-6 of the table's
largest entry (columns that are mathematically zero, such as the mean velocity and the
net transfer sums, hold FP32 rounding noise).
"""
import numpy as np
import pytest

from oracle.ffs_oracle import OracleSimulation, Params

pytestmark = pytest.mark.gpu

FIELD_TOL = 2e-6
STATS_TOL = 1e-5


def gdict(n, **kw):
    d = {"nx": str(n), "ny": str(n), "nz": str(n), "xDomainSize": "1.0", "yDomainSize": "1.0",
         "zDomainSize": "1.0", "kinematicViscosity": "1e-3", "dtStat": "1", "dtSpec": "2", "writeTime": "1000",
         "velocityTimeStep": "Adams_Bashforth3rdO", "variableTimestepFlag": "true", "cfl": "0.5", "dt": "0.001",
         "forcing": "isotropicBand", "forcingPower": "0.1", "forcingKf": "2.5"}
    d.update({k: str(v) for k, v in kw.items()})
    return d


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def make(pkg, d, u, variant):
    p = pkg.parameters(d, precision="FP32")
    p.kernel_variant = variant
    sim = pkg.Simulation(p)
    sim.set_fields(*u)
    sim.initialize()
    return sim


@pytest.mark.parametrize("n,dtstat,variant", [(64, 1, 0), (128, 1, 0), (256, 1, 0), (256, 1000, 0), (512, 2, 0),
                                               (128, 1, 2), (256, 1, 2), (512, 2, 2), (128, 1, 3), (256, 1, 3)])
def test_fused_matches_generic(gpu_pkg, n, dtstat, variant):
    d = gdict(n, dtStat=dtstat)
    u = gpu_pkg.random_spectrum(n, k0=4.0, seed=11)
    a, b = make(gpu_pkg, d, u, variant), make(gpu_pkg, d, u, 1)
    steps = 5 if n < 512 else 3
    a.advance_in_time(steps)
    b.advance_in_time(steps)
    for c in range(3):
        assert rel(a.spectral(c), b.spectral(c)) <= FIELD_TOL, (n, c)
    assert a.dt == pytest.approx(b.dt, rel=1e-6)
    ra, rb = a.stats_rows(), b.stats_rows()
    assert ra.shape == rb.shape and ra.shape[0] >= 1
    assert (np.abs(ra - rb) <= STATS_TOL * np.abs(rb) + 1e-6 * np.abs(rb).max()).all()
    a.close()
    b.close()


def test_fused_fp32_against_oracle(gpu_pkg):
    """128^3 forced DNS, adaptive AB3: FP32 (fused x pass) within 1e-4 of the FP64 oracle
    after 10 steps."""
    n = 128
    d = gdict(n, dtStat=5, dtSpec=1000)
    u = gpu_pkg.random_spectrum(n, k0=4.0, seed=12)
    sim = make(gpu_pkg, d, u, 0)
    sim.advance_in_time(10)
    ref = OracleSimulation(Params.from_global(d), u)
    ref.initialize()
    ref.run(10)
    for c in range(3):
        assert rel(sim.spectral(c), ref.u[c]) <= 1e-4, c
    sim.close()


def les_dict(n, den):
    d = {"nx": str(n), "ny": str(n), "nz": str(n), "xDomainSize": "1.0", "yDomainSize": "1.0",
         "zDomainSize": "1.0", "kinematicViscosity": "5e-4", "dtStat": "1", "dtSpec": "2", "writeTime": "1000",
         "velocityTimeStep": "ETD3rdO", "variableTimestepFlag": "true", "cfl": "0.18", "dt": "0.001",
         "lesModel": "Smagorinsky", "smagorinskyConstant": "0.17", "filterWidth": repr(2 * np.pi / n)}
    if den:
        d.update({"densityStratification": "true", "zAcceleration": "1", "referenceDensity": "1",
                  "densityGradient": "1", "Pr": "1"})
    return d


@pytest.mark.parametrize("n,den,variant", [(64, False, 0), (128, False, 0), (64, True, 0), (128, True, 0),
                                           (128, True, 3)])
def test_les_fused_matches_generic(gpu_pkg, n, den, variant):
    """The twelve-field register-fused x pass (Smagorinsky LES, with and without
    Boussinesq density; n = 64, 128) and the line-pair forward z pass with the stress and
    flux fields (128; variant 3: one line per thread) against the generic kernels."""
    d = les_dict(n, den)
    u = gpu_pkg.random_spectrum(n, k0=3.0, seed=13)
    sims = []
    for variant in (variant, 1):
        p = gpu_pkg.parameters(d, precision="FP32")
        p.kernel_variant = variant
        sim = gpu_pkg.Simulation(p)
        sim.set_fields(*u, rho=np.zeros_like(u[0]) if den else None)
        sim.initialize()
        sim.advance_in_time(5)
        sims.append(sim)
    a, b = sims
    for c in range(3):
        assert rel(a.spectral(c), b.spectral(c)) <= FIELD_TOL, (n, c)
    if den:   # rho starts at zero and grows from its source term over the 5 steps, so the
        # two FP32 operation orders differ by ~2e-6 of it; the bar is 1e-5
        assert rel(a.spectral(3), b.spectral(3)) <= 1e-5, n
    assert a.dt == pytest.approx(b.dt, rel=1e-6)
    ra, rb = a.stats_rows(), b.stats_rows()
    assert ra.shape == rb.shape and ra.shape[0] >= 1
    assert (np.abs(ra - rb) <= STATS_TOL * np.abs(rb) + 1e-6 * np.abs(rb).max()).all()
    a.close()
    b.close()
