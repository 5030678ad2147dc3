"""Parity of the CUDA engine (through the C ABI) with the FP64 CPU oracle.

Tolerances: FP64 fields 1e-12 relative L2 per component after 10 steps, FP64 stats rows
1e-10 relative; FP32 fields 1e-4 relative L2 after 10 steps. Adaptive-dt ETD runs are
an exception (see test_etd_adaptive_parity): their dt comes from a max over FFT output,
which differs from any other FFT in the last bit, and the reference's own ETD
coefficient formulas amplify such a difference ~1e7 times.
"""
import numpy as np
import pytest

from oracle.ffs_oracle import Grid, OracleSimulation, Params, stats_header

pytestmark = pytest.mark.gpu

FP64_FIELD_TOL = 1e-12
FP64_STATS_TOL = 1e-10
FP32_FIELD_TOL = 1e-4


def gdict(n, integ="Adams_Bashforth3rdO", adaptive=False, dt="0.01", ny=None, nz=None, **kw):
    d = {"nx": str(n), "ny": str(ny or n), "nz": str(nz or n), "xDomainSize": "1.0", "yDomainSize": "1.0",
         "zDomainSize": "1.0", "kinematicViscosity": "0.01", "dtStat": "2", "dtSpec": "3", "writeTime": "1000",
         "velocityTimeStep": integ, "variableTimestepFlag": "true" if adaptive else "false", "cfl": "0.5",
         "dt": dt}
    d.update({k: str(v) for k, v in kw.items()})
    return d


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / nb if nb > 0 else np.linalg.norm(a - b)


def make_ic(pkg, d, seed=7, k0=3.0, density=False):
    nx, ny, nz = int(d["nx"]), int(d["ny"]), int(d["nz"])
    if nx == ny == nz:
        u = pkg.random_spectrum(nx, k0=k0, seed=seed)
    else:
        rng = np.random.default_rng(seed)
        g = Grid(nx, ny, nz)
        uh = np.stack([g.myfourier(rng.standard_normal((nz, ny, nx))) for _ in range(3)])
        uh = g.project(uh) * np.exp(-np.sqrt(g.K2) / 4)[None]
        u = tuple(g.real(uh))
    rho = None
    if density and nx == ny == nz:
        rho = 0.1 * pkg.random_spectrum(nx, k0=k0, seed=seed + 1)[0]
    elif density:
        rng = np.random.default_rng(seed + 1)
        g = Grid(nx, ny, nz)
        rh = g.myfourier(rng.standard_normal((nz, ny, nx))) * np.exp(-np.sqrt(g.K2) / 4)
        rh[0, 0, 0] = 0.0
        rho = 0.1 * g.real(rh) / np.sqrt(np.mean(g.real(rh) ** 2))
    return u, rho


def run_pair(pkg, d, steps=10, precision="FP64", seed=7, density=False):
    u, rho = make_ic(pkg, d, seed=seed, density=density)
    sim = pkg.Simulation.from_global(d, precision=precision)
    sim.set_fields(*u, rho)
    sim.initialize()
    sim.advance_in_time(steps)
    ref = OracleSimulation(Params.from_global(d), u, rho)
    ref.initialize()
    ref.run(steps)
    return sim, ref


FIXED_CASES = {
    "ab3-32": gdict(32),
    "ab3-48-radix3": gdict(48),
    "ab3-64-hv-forced": gdict(64, hyperViscosity="true", hyperViscosityCoefficient="1e-6",
                              forcing="isotropicBand", forcingPower="0.1", forcingKf="2.5"),
    "ab3-noncubic": gdict(32, ny=48, nz=64),
    "etd-32": gdict(32, "ETD3rdO"),
    "etd-96": gdict(96, "ETD3rdO", dt="0.005"),
    "etd-les-density": gdict(32, "ETD3rdO", lesModel="Smagorinsky", densityStratification="true", Pr="1",
                             densityGradient="1", zAcceleration="1", referenceDensity="1"),
    "etd-hv-L2": gdict(32, "ETD3rdO", hyperViscosity="true", hyperViscosityCoefficient="1e-5",
                       xDomainSize="2.0", yDomainSize="2.0", zDomainSize="2.0"),
    "ab3-adaptive": gdict(32, adaptive=True),
    # nz >= 128: the forward z pass runs one component at a time
    "etd-128-les-density": gdict(128, "ETD3rdO", dt="0.002", lesModel="Smagorinsky", densityStratification="true",
                                 Pr="1", densityGradient="1", zAcceleration="1", referenceDensity="1"),
    "ab3-adaptive-density": gdict(32, adaptive=True, densityStratification="true", Pr="2", densityGradient="1",
                                  zAcceleration="1", referenceDensity="1"),
    # the other pointwise LES models of les_types (les_types.jl:360-395)
    "etd-vreman": gdict(32, "ETD3rdO", lesModel="Vreman", vremanConstant="0.07"),
    "ab3-production-viscosity": gdict(32, lesModel="productionViscosity"),
    "etd-silvis": gdict(32, "ETD3rdO", lesModel="Silvis"),
    "ab3-stable-nonlinear": gdict(32, lesModel="stableNonLinear", nlConstant="0.05"),
    "etd-sandp-smagorinsky": gdict(32, "ETD3rdO", lesModel="SandP", sLesModel="Smagorinsky"),
    # the dynamic Smagorinsky model (dynamic_smagorinsky.jl): full-spectrum test filter of
    # Sa and L, Germano coefficient, filtered again; radix-2, radix-3 and non-cubic grids
    "etd-dynamic-smagorinsky": gdict(32, "ETD3rdO", lesModel="dynamicSmagorinsky"),
    "ab3-dynamic-48-cmin-density": gdict(48, lesModel="dynamicSmagorinsky", TestFilterWidth="0.4", cmin="-0.05",
                                         densityStratification="true", Pr="1", densityGradient="1",
                                         zAcceleration="1", referenceDensity="1"),
    "etd-dynamic-noncubic": gdict(32, "ETD3rdO", ny=48, nz=64, lesModel="dynamicSmagorinsky", filterWidth="0.3"),
    # piomelliSmagorinsky: the previous coefficient extrapolated in time (adaptive dt makes
    # dt/dtm1 vary), c = (tau^ + L):M/M:M
    "ab3-adaptive-piomelli": gdict(32, adaptive=True, lesModel="piomelliSmagorinsky"),
    "etd-piomelli-48-cmin": gdict(48, "ETD3rdO", lesModel="piomelliSmagorinsky", cmin="-0.05",
                                  TestFilterWidth="0.35"),
    # the dynamic P tensor term (dynamicSandP / piomelliSandP) on either dynamic model
    "etd-dynamic-sandp": gdict(32, "ETD3rdO", lesModel="dynamicSandP", sLesModel="dynamicSmagorinsky"),
    "ab3-adaptive-piomelli-sandp": gdict(32, adaptive=True, lesModel="piomelliSandP", sLesModel="piomelliSmagorinsky"),
    "ab3-adaptive-piomellip-dynamic": gdict(32, adaptive=True, lesModel="piomelliSandP",
                                            sLesModel="dynamicSmagorinsky"),
    "etd-48-dynamicsandp-piomelli": gdict(48, "ETD3rdO", lesModel="dynamicSandP", sLesModel="piomelliSmagorinsky",
                                          cmin="-0.02"),
    "ab3-sandp-dynamic": gdict(32, lesModel="SandP", sLesModel="dynamicSmagorinsky", pConstant="0.12"),
    # the spectral barrier (hyperviscosity_types.jl:32-82, ETD.jl:71-82) and the density's
    # own hyperviscosity (density_stratification_types.jl:137-148; AB3 adds no term)
    "etd-spectral-barrier": gdict(32, "ETD3rdO", hyperViscosity="spectralBarrier"),
    "etd-barrier-truncating": gdict(32, "ETD3rdO", hyperViscosity="spectralBarrier", initk="5", endk="20"),
    "etd-density-hv": gdict(32, "ETD3rdO", densityStratification="true", Pr="1", densityGradient="1",
                            zAcceleration="1", referenceDensity="1", densityHyperViscosity="true",
                            densityHyperViscosityCoefficient="1e-5"),
    "ab3-adaptive-density-hv": gdict(32, adaptive=True, densityStratification="true", Pr="2", densityGradient="1",
                                     zAcceleration="1", referenceDensity="1", densityHyperViscosity="true",
                                     densityHyperViscosityCoefficient="1e-4", densityHyperViscosityM="3"),
    "etd-barriers-density-specfil": gdict(32, "ETD3rdO", hyperViscosity="spectralBarrier", densityStratification="true",
                                          Pr="1", densityGradient="1", zAcceleration="1", referenceDensity="1",
                                          densityHyperViscosity="spectralBarrier", densityInitk="6", specFil="2"),
    "etd-scalar-barrier": gdict(32, "ETD3rdO", passiveScalar="true", scalarPr="0.7", scalarGradient="1",
                                hyperViscosity="spectralBarrier", initk="6"),
    # the reference's kz = 0 plane forcing family (forcing_types.jl:335-450)
    "ab3-adaptive-rf-forcing": gdict(32, adaptive=True, forcing="rfForcing", TF="2.0", alphac="1.0", kf="3.0"),
    "etd-crf-forcing-tanh": gdict(32, "ETD3rdO", forcing="cRfForcing", TF="0.5", alphac="1.0", kf="4.0", Zf="tanh"),
    "ab3-adaptive-qf-forcing-les": gdict(32, adaptive=True, forcing="QfForcing", alveliusP="0.1", alveliusC="1.0",
                                         alveliusKf="2.0", kf="4.0", lesModel="Smagorinsky"),
    "ab3-adaptive-nrf-forcing": gdict(32, adaptive=True, forcing="nRfForcing", TF="2.0", alphac="1.0", kf="3.0"),
    "etd-cnrf-forcing-les": gdict(32, "ETD3rdO", forcing="cNRfForcing", TF="0.5", alphac="1.0", kf="3.0",
                                  lesModel="Smagorinsky"),
    "ab3-a-forcing-tanh": gdict(32, forcing="aForcing", TF="2.0", alphac="1.0", kf="3.0", Zf="tanh"),
    # passive scalar (simulationtypes.jl:198-213): the density's transport without buoyancy
    "etd-scalar": gdict(32, "ETD3rdO", passiveScalar="true", scalarPr="0.7", scalarGradient="1"),
    "ab3-adaptive-scalar-y": gdict(32, adaptive=True, passiveScalar="true", scalarPr="2", scalarGradient="0.5",
                                   scalarDirection="y"),
    # the scalar's ETD takes the velocity's hyperviscosity (simulationtypes.jl:336)
    "etd-scalar-hv": gdict(32, "ETD3rdO", passiveScalar="true", scalarPr="1", scalarGradient="1",
                           hyperViscosity="true", hyperViscosityCoefficient="1e-5"),
    "ab3-sandp-vreman-density": gdict(48, lesModel="SandP", sLesModel="Vreman", densityStratification="true",
                                      Pr="1", densityGradient="1", zAcceleration="1", referenceDensity="1"),
    # specFil (Globals.jl:173-182): the Stats_fil.txt row beside every Stats.txt row, and
    # the reference's STAT_FIL side effects on Stats.txt (pressure columns) and on the
    # CFL slot (adaptive cases)
    "etd-les-density-hv-specfil": gdict(32, "ETD3rdO", lesModel="Smagorinsky", densityStratification="true", Pr="1",
                                        densityGradient="1", zAcceleration="1", referenceDensity="1",
                                        hyperViscosity="true", hyperViscosityCoefficient="1e-5", specFil="2"),
    "ab3-adaptive-density-specfil": gdict(32, adaptive=True, densityStratification="true", Pr="2", densityGradient="1",
                                          zAcceleration="1", referenceDensity="1", specFil="3"),
    "ab3-adaptive-scalar-specfil": gdict(32, adaptive=True, passiveScalar="true", scalarPr="0.7", scalarGradient="1",
                                         specFil="1.5", forcing="isotropicBand", forcingPower="0.1", forcingKf="2.5"),
    # LES of the density and the scalar (les_real_calc.jl:116-134): eddy diffusion nu_t grad rho,
    # vorticity diffusion + (c D^2 / 2) w x grad rho; nu_t of each model; rhopr and its
    # place in trhodiss and in the CFL slots (density_stratification_types.jl:46-87)
    "etd-les-density-eddy": gdict(32, "ETD3rdO", lesModel="Smagorinsky", densityStratification="true", Pr="1",
                                  densityGradient="1", zAcceleration="1", referenceDensity="1",
                                  densityLesModel="eddyDiffusion"),
    "etd-dynamic-density-vorticity": gdict(32, "ETD3rdO", lesModel="dynamicSmagorinsky", densityStratification="true",
                                           Pr="1", densityGradient="1", zAcceleration="1", referenceDensity="1",
                                           densityLesModel="vorticityDiffusion", densityVorticityCoefficient="0.3"),
    "ab3-adaptive-vreman-density-vort-specfil": gdict(32, adaptive=True, lesModel="Vreman", densityStratification="true",
                                                      Pr="2", densityGradient="1", zAcceleration="1",
                                                      referenceDensity="1", densityLesModel="vorticityDiffusion",
                                                      specFil="2"),
    "ab3-adaptive-stablenl-density-eddy-hv": gdict(32, adaptive=True, lesModel="stableNonLinear",
                                                   densityStratification="true", Pr="1", densityGradient="1",
                                                   zAcceleration="1", referenceDensity="1",
                                                   densityLesModel="eddyDiffusion", densityHyperViscosity="true",
                                                   densityHyperViscosityCoefficient="1e-4"),
    "ab3-production-density-eddy": gdict(48, lesModel="productionViscosity", densityStratification="true", Pr="1",
                                         densityGradient="1", zAcceleration="1", referenceDensity="1",
                                         densityLesModel="eddyDiffusion"),
    "etd-scalar-les": gdict(32, "ETD3rdO", lesModel="Smagorinsky", passiveScalar="true", scalarPr="0.7",
                            scalarGradient="1"),
    "ab3-adaptive-silvis-scalar-vort": gdict(32, adaptive=True, lesModel="Silvis", passiveScalar="true", scalarPr="1",
                                             scalarGradient="1", scalarLesModel="vorticityDiffusion",
                                             scalarVorticityCoefficient="0.5"),
    # Euller (Euller.jl): u += dt rhs with the explicit viscosity, dt as set_dt! gives it
    "euler-32": gdict(32, "Euller", dt="0.005"),
    "euler-adaptive-les-density-eddy": gdict(32, "Euller", adaptive=True, lesModel="Smagorinsky",
                                             densityStratification="true", Pr="1", densityGradient="1",
                                             zAcceleration="1", referenceDensity="1", densityLesModel="eddyDiffusion"),
    "euler-scalar-forced": gdict(32, "Euller", dt="0.005", passiveScalar="true", scalarPr="0.7", scalarGradient="1",
                                 forcing="rfForcing", TF="2.0", alphac="1.0", kf="3.0"),
    # nz >= 128: the flux's z component comes from the density's slot on the one-component path
    "etd-nz128-les-density-vort": gdict(32, "ETD3rdO", nz=128, dt="0.005", lesModel="Smagorinsky",
                                        densityStratification="true", Pr="1", densityGradient="1", zAcceleration="1",
                                        referenceDensity="1", densityLesModel="vorticityDiffusion"),
}


@pytest.mark.parametrize("name", sorted(FIXED_CASES))
def test_fp64_step_parity(gpu_pkg, name):
    d = FIXED_CASES[name]
    fld = "densityStratification" in d or "passiveScalar" in d
    sim, ref = run_pair(gpu_pkg, d, density=fld)
    for c in range(3):
        assert rel(sim.spectral(c), ref.u[c]) <= FP64_FIELD_TOL, (name, c)
    if fld:
        assert rel(sim.spectral(3), ref.rho) <= FP64_FIELD_TOL
    recs = sim.records()                 # reading drains the pending records
    rows = recs[:, : sim.ncols]
    rr = np.array(ref.stats_rows)
    assert rows.shape == rr.shape
    assert sim.header.count(",") + 1 == rows.shape[1]
    assert sim.header == stats_header(Params.from_global(d))
    # relative error per entry, with an absolute floor of 1e-6 x the table's largest entry
    # for columns that are mathematically zero (mean velocity, net transfer: ~1e-20 noise)
    scale = np.maximum(np.abs(rr), 1e-6 * np.abs(rr).max())
    err = np.abs(rows - rr) / scale
    assert err.max() <= FP64_STATS_TOL, (name, np.unravel_index(err.argmax(), err.shape), err.max())
    assert sim.has_stats_fil == ("specFil" in d)
    if sim.has_stats_fil:   # Stats_fil.txt rows, same bar
        fr, fe = sim.stats_fil_rows(recs), np.array(ref.stats_fil_rows)
        assert fr.shape == fe.shape == rr.shape
        scale = np.maximum(np.abs(fe), 1e-6 * np.abs(fe).max())
        err = np.abs(fr - fe) / scale
        assert err.max() <= FP64_STATS_TOL, (name, "fil", np.unravel_index(err.argmax(), err.shape), err.max())
    assert sim.iteration == ref.iteration
    assert sim.time == pytest.approx(ref.time, rel=1e-14)
    sim.close()


def test_etd_adaptive_parity(gpu_pkg):
    """Adaptive ETD: dt = cfl dx / max|u| follows the FFT output; a last-bit difference in
    dt changes the rounding of the reference's cancelling phi formulas (ETD.jl:181-191),
    so the bar here is the oracle's own sensitivity: 1e-8 after 10 steps."""
    d = gdict(32, "ETD3rdO", adaptive=True)
    sim, ref = run_pair(gpu_pkg, d)
    for c in range(3):
        assert rel(sim.spectral(c), ref.u[c]) <= 1e-8
    assert sim.dt == pytest.approx(ref.get_dt(), rel=1e-13)


@pytest.mark.parametrize("name", ["ab3-32", "etd-les-density", "ab3-64-hv-forced", "etd-vreman", "etd-silvis",
                                  "ab3-stable-nonlinear", "etd-dynamic-smagorinsky", "ab3-adaptive-piomelli",
                                  "ab3-adaptive-piomelli-sandp", "etd-les-density-eddy",
                                  "ab3-adaptive-silvis-scalar-vort", "euler-adaptive-les-density-eddy"])
def test_fp32_error(gpu_pkg, name):
    d = FIXED_CASES[name]
    sim, ref = run_pair(gpu_pkg, d, precision="FP32", density="densityStratification" in d)
    for c in range(3):
        assert rel(sim.spectral(c), ref.u[c]) <= FP32_FIELD_TOL, (name, c)
    sim.close()


def test_transform_roundtrip(gpu_pkg):
    """set_fields = myfourier! (utils.jl:101-106); get_fields = real! (unnormalised c2r)."""
    n = 48
    d = gdict(n)
    u, _ = make_ic(gpu_pkg, d)
    g = Grid(n, n, n)
    for prec, tol in (("FP64", 1e-14), ("FP32", 1e-6)):
        sim = gpu_pkg.Simulation.from_global(d, precision=prec)
        rng = np.random.default_rng(3)
        raw = [rng.standard_normal((n, n, n)) for _ in range(3)]
        sim.set_fields(*raw)
        for c in range(3):
            assert rel(sim.spectral(c), g.myfourier(raw[c])) <= tol
        f = sim.fields()
        for c in range(3):
            assert rel(f[c], g.real(g.myfourier(raw[c]))) <= tol
        # padded layout round trip
        fp = sim.fields(layout=1)
        assert fp[0].shape == (n, n, 2 * (n // 2 + 1))
        assert np.array_equal(fp[0][:, :, :n], f[0]) and not fp[0][:, :, n:].any()
        sim.close()


SPEC_CASES = {
    "ab3": gdict(32, dtSpec="2"),
    "etd-les-density": dict(FIXED_CASES["etd-les-density"], dtSpec="2"),
    "ab3-hv-forced": dict(FIXED_CASES["ab3-64-hv-forced"], dtSpec="2"),
    "etd-scalar": dict(FIXED_CASES["etd-scalar"], dtSpec="2"),
    "etd-les-density-hv-specfil": dict(FIXED_CASES["etd-les-density-hv-specfil"], dtSpec="2"),
    "etd-barriers-density-specfil": dict(FIXED_CASES["etd-barriers-density-specfil"], dtSpec="2"),
    "etd-dynamic-density-vorticity": dict(FIXED_CASES["etd-dynamic-density-vorticity"], dtSpec="2"),
    # write_spec_forcing (spec.jl:148-170): the forcing spectrum of the kz = 0 plane family
    "ab3-adaptive-rf-forcing": dict(FIXED_CASES["ab3-adaptive-rf-forcing"], dtSpec="2"),
    "ab3-a-forcing-tanh": dict(FIXED_CASES["ab3-a-forcing-tanh"], dtSpec="2"),
}


@pytest.mark.parametrize("name", sorted(SPEC_CASES))
def test_spectrum_parity(gpu_pkg, name):
    """Every write_spec spectrum (spec.jl:1-146, 196-450) against the oracle, FP64."""
    d = SPEC_CASES[name]
    density = "densityStratification" in d or "passiveScalar" in d
    sim, ref = run_pair(gpu_pkg, d, steps=5, density=density)
    got = sim.spectra()
    assert [r["iteration"] for r in got] == sorted(ref.spectra)
    fields = sim.spectrum_fields
    assert fields[:8] == ["u_h", "u_v", "vis_h", "vis_v", "nl_h", "nl_v", "press_h", "press_v"]
    for r in got:
        e = ref.spectra[r["iteration"]]
        keys = [f"{f}.{s}" for f in fields for s in ("specH", "specV")] + ["u.specH"]
        for key in keys:
            # transfer spectra sum to ~0: the floor is relative to the field's own scale
            scale = max(np.abs(e[key]).max(), 1e-300)
            assert np.allclose(r[key], e[key], rtol=1e-10, atol=1e-12 * scale), (name, key)
    sim.close()


def test_errors_and_state_checks(gpu_pkg):
    d = gdict(32)
    sim = gpu_pkg.Simulation.from_global(d)
    with pytest.raises(gpu_pkg.FFSError) as e:
        sim.advance_in_time(1)           # before initialize
    assert e.value.code == -7
    bad = dict(d, nx="40")
    with pytest.raises(gpu_pkg.FFSError) as e:
        gpu_pkg.Simulation.from_global(bad)
    assert e.value.code == -6
    # the reference's AB3 has no explicit term for the spectral barrier
    with pytest.raises(gpu_pkg.FFSError) as e:
        gpu_pkg.Simulation.from_global(dict(d, hyperViscosity="spectralBarrier"))
    assert e.value.code == -6
    # the density's LES diffusion needs an LES model (the reference's flux would keep a bare
    # grad rho): refused through the C ABI too
    prm = gpu_pkg.parameters(dict(d, densityStratification="true", Pr="1", densityGradient="1",
                                  zAcceleration="1", referenceDensity="1"))
    prm.rho_les = 1
    with pytest.raises(gpu_pkg.FFSError) as e:
        gpu_pkg.Simulation(prm)
    assert e.value.code == -6
    # nRfForcing reads the integrator's dt2, which Euller does not keep (nrforcing.jl:37)
    with pytest.raises(gpu_pkg.FFSError) as e:
        gpu_pkg.Simulation.from_global(dict(d, velocityTimeStep="Euller", forcing="nRfForcing", TF="2.0",
                                            alphac="1.0", kf="3.0"))
    assert e.value.code == -6
    # a non-finite initial condition is reported, not propagated silently
    u, _ = make_ic(gpu_pkg, d)
    u = [x.copy() for x in u]
    u[0][3, 4, 5] = np.nan
    sim.set_fields(*u)
    sim.initialize()
    with pytest.raises(gpu_pkg.FFSError) as e:
        sim.advance_in_time(2)
    assert e.value.code == -4
    sim.close()


def test_restart_continues_like_one_run(gpu_pkg):
    """Two step calls of 4 and 6 equal one call of 10 (graph replay keeps all state on the device)."""
    d = gdict(32, "ETD3rdO")
    u, _ = make_ic(gpu_pkg, d)
    a = gpu_pkg.Simulation.from_global(d)
    a.set_fields(*u)
    a.initialize()
    a.advance_in_time(10)
    b = gpu_pkg.Simulation.from_global(d)
    b.set_fields(*u)
    b.initialize()
    b.advance_in_time(4)
    b.advance_in_time(6)
    for c in range(3):
        assert np.array_equal(a.spectral(c), b.spectral(c))
    assert np.array_equal(a.stats_rows(), b.stats_rows())


def test_full_size_properties(gpu_pkg):
    """256^3 FP32 forced DNS: divergence-free, finite, energy budget consistent."""
    n = 256
    d = gdict(n, adaptive=True, kinematicViscosity="1e-3", forcing="isotropicBand", dtStat="1", dtSpec="1000")
    u = gpu_pkg.random_spectrum(n, k0=4.0, seed=2001)
    sim = gpu_pkg.Simulation.from_global(d, precision="FP32")
    sim.set_fields(*u)
    sim.initialize()
    sim.advance_in_time(6)
    g = Grid(n, n, n)
    uh = [sim.spectral(c) for c in range(3)]
    div = g.KX * uh[0] + g.KY * uh[1] + g.KZ * uh[2]
    assert np.abs(div).max() <= 1e-5 * max(np.abs(x).max() for x in uh)
    rows = sim.stats_rows()
    assert np.isfinite(rows).all()
    k = rows[:, 11]
    assert abs(k[0] - 1.5) < 1e-3            # u_rms = 1 -> k = 3/2
    # dealiased nonlinear transfer conserves energy: nl + press ~ 0 relative to dissipation
    assert np.abs(rows[:, 15] + rows[:, 16] + rows[:, 17] + rows[:, 18]).max() < 1e-3 * rows[:, 14].max()
    sim.close()


@pytest.mark.parametrize("name", ["ab3-32", "etd-les-density", "ab3-64-hv-forced"])
def test_scales_and_numbers_parity(gpu_pkg, name):
    """Scales.txt / Numbers.txt rows (stats.jl:64-165) from the engine's records against
    the oracle's direct evaluation on its spectral state."""
    d = FIXED_CASES[name]
    sim, ref = run_pair(gpu_pkg, d, density="densityStratification" in d)
    sc, nums = sim.scales_numbers(sim.records())
    for got, want in ((np.array(sc), np.array(ref.scales_rows)), (np.array(nums), np.array(ref.numbers_rows))):
        assert got.shape == want.shape and got.shape[0] >= 2
        ok = np.isfinite(want)
        assert np.array_equal(ok, np.isfinite(got))
        scale = np.maximum(np.abs(want[ok]), 1e-6 * np.abs(want[ok]).max())
        assert (np.abs(got[ok] - want[ok]) / scale).max() <= FP64_STATS_TOL, name
    sim.close()


@pytest.mark.parametrize("precision,tol", [("FP64", 1e-10), ("FP32", 1e-4)])
def test_current_stats_and_spectrum(gpu_pkg, precision, tol):
    """ffs_stats (the latest Stats.txt row, left in the pending records) and ffs_spectrum
    (u spectrum of the current state: u.specH and u_h.specV + u_v.specV) against the
    drained rows and the oracle's spectrum_u of the same state."""
    d = gdict(32, integ="ETD3rdO", dtStat=1)
    u, _ = make_ic(gpu_pkg, d)
    sim = gpu_pkg.Simulation.from_global(d, precision=precision)
    sim.set_fields(*u)
    sim.initialize()
    with pytest.raises(gpu_pkg.FFSError):   # no stats iteration yet
        sim.stats()
    sim.advance_in_time(3)
    last = sim.stats()
    rows = sim.stats_rows()
    assert rows.shape[0] == 3 and np.array_equal(last, rows[-1])
    H, V = sim.spectrum()
    ref = OracleSimulation(Params.from_global(d), u)
    ref.initialize()
    ref.run(3)
    sp = ref.spectrum_u()
    assert rel(H, sp["u.specH"]) <= tol
    assert rel(V, sp["u_h.specV"] + sp["u_v.specV"]) <= tol
    sim.close()


# Every alternative radix split the autotuner may pick for the runtime-plan passes
# (ffs_params.radix_split forces it on every axis that has one), FP64 against the oracle
# at the usual bars; non-cubic grids mix axes with and without the split.
RADIX_CASES = [(gdict(32), 1), (gdict(32), 2), (gdict(48, "ETD3rdO"), 1), (gdict(48), 2),
               (gdict(64, lesModel="Smagorinsky"), 1), (gdict(64), 2), (gdict(96, "ETD3rdO", dt="0.005"), 1),
               (gdict(96), 2), (gdict(128), 1), (gdict(128, "ETD3rdO", dt="0.005"), 2), (gdict(32, ny=48, nz=64), 2),
               (gdict(16, ny=32, nz=48), 1)]


@pytest.mark.parametrize("case", range(len(RADIX_CASES)))
def test_radix_split_parity(gpu_pkg, case):
    d, split = RADIX_CASES[case]
    u, rho = make_ic(gpu_pkg, d)
    p = gpu_pkg.parameters(d, precision="FP64")
    p.radix_split = split
    sim = gpu_pkg.Simulation(p)
    sim.set_fields(*u, rho)
    sim.initialize()
    sim.advance_in_time(10)
    ref = OracleSimulation(Params.from_global(d), u, rho)
    ref.initialize()
    ref.run(10)
    for c in range(3):
        assert rel(sim.spectral(c), ref.u[c]) <= FP64_FIELD_TOL, (case, c)
    rows, rr = sim.stats_rows(), np.array(ref.stats_rows)
    scale = np.maximum(np.abs(rr), 1e-6 * np.abs(rr).max())
    assert (np.abs(rows - rr) / scale).max() <= FP64_STATS_TOL
    sim.close()


def test_radix_split_fp32_runtime_plans(gpu_pkg):
    """FP32 with runtime-plan kernels only (kernel_variant 1) on an alternative split."""
    d = gdict(128)
    u, rho = make_ic(gpu_pkg, d)
    p = gpu_pkg.parameters(d, precision="FP32")
    p.kernel_variant = 1
    p.radix_split = 1
    sim = gpu_pkg.Simulation(p)
    sim.set_fields(*u, rho)
    sim.initialize()
    sim.advance_in_time(10)
    ref = OracleSimulation(Params.from_global(d), u, rho)
    ref.initialize()
    ref.run(10)
    for c in range(3):
        assert rel(sim.spectral(c), ref.u[c]) <= FP32_FIELD_TOL
    sim.close()
