"""File-level drop-in test: ``run_simulation()`` on a case directory (a `global` file and
u1.0/u2.0/u3.0) against the oracle run the way the reference's run_simulation runs it
(src/FluidFlowSimulation.jl:23-65).

Compared, FP64: every Stats.txt, Scales.txt and Numbers.txt line (1e-10), every
spectrum file (1e-10), and the u1.N/u2.N/u3.N files (sizes 8 nx ny nz bytes, contents
1e-12 relative L2). The oracle side restates the loop: the fields are written from
calculate_rhs! when a step starts at a multiple of writeTime (is_output_time,
src/simulationtypes.jl:102, src/models.jl:158) and once more at the end; the tail runs
calculate_rhs!, the forcing and writestats at the final iteration.
"""
import math

import numpy as np
import pytest

from oracle.ffs_oracle import OracleSimulation, Params, stats_header

pytestmark = pytest.mark.gpu


def forcing_files(s):
    """writeoutput's kz = 0 forcing arrays (output.jl:45-67) of the oracle's forcing now."""
    f, kind = s.pforce, s.p.plane_forcing
    if kind == "aForcing":
        return {"R": f.R2.T.copy()}                     # the reference's R[kx, y]
    if kind in ("rfForcing", "cRfForcing", "nRfForcing", "cNRfForcing"):
        out = {"R": f.R.copy(), "Eh": np.stack([f.kh, f.Ef], 1)}
        if kind in ("nRfForcing", "cNRfForcing"):
            out["N"] = f.N.copy()
        return out
    return {}


def oracle_run(d, u):
    """FluidFlowSimulation.jl:23-65 on the oracle; returns its rows, spectra and outputs:
    the u fields, the LES fields captured by the calculate_rhs! at each output iteration
    (T11..T23, cs, cp, dflux) and the forcing files."""
    s = OracleSimulation(Params.from_global(d), u)
    total = int(d["nt"]) if "nt" in d else (1 << 62)
    lengthtime = float(d["timeDuration"]) if "timeDuration" in d else math.inf
    wt = int(d["writeTime"])
    s.initialize()
    final, finaltime = s.iteration + total, s.time + lengthtime
    outputs, les, forcing = {}, {}, {}
    calls = 0                                    # the integrator's call count
    while s.iteration < final and s.time < finaltime:
        out_step = calls != 0 and s.iteration % wt == 0
        it = s.iteration
        if out_step:
            outputs[it] = s.u_physical()
            forcing[it] = forcing_files(s)
        s.advance()
        if out_step and s.p.les:
            les[it] = dict(s.les_out)
        calls += 1
    in_rhs = calls != 0 and s.iteration % wt == 0
    pre = forcing_files(s)
    s.finalize()                                 # calculate_rhs!, forcing, writestats
    outputs[s.iteration] = s.u_physical()        # tail calculate_rhs! or the explicit writeoutput
    forcing[s.iteration] = pre if in_rhs else forcing_files(s)
    if s.p.plane_forcing == "rfForcing":         # FluidFlowSimulation.jl:60-62 rewrites R.N last
        forcing[s.iteration]["R"] = s.pforce.R.copy()
    if s.p.les:
        les[s.iteration] = dict(s.les_out)
    return s, outputs, les, forcing


def read_rows(path):
    lines = path.read_text().splitlines()
    return lines[0], np.array([[float(x) for x in ln.split(",")] for ln in lines[1:]])


def rows_err(got, want):
    got, want = np.asarray(got), np.asarray(want)
    assert got.shape == want.shape, (got.shape, want.shape)
    ok = np.isfinite(want)
    assert np.array_equal(ok, np.isfinite(got))
    scale = np.maximum(np.abs(want[ok]), 1e-6 * np.abs(want[ok]).max())
    return float((np.abs(got[ok] - want[ok]) / scale).max())


CASES = {
    # ETD3, fixed dt, band forcing: stats at 0,3,6,9 + the tail at 12, spectra at 0,4,8,12,
    # fields at 5, 10 and 12
    "etd-forced-nt": {"velocityTimeStep": "ETD3rdO", "variableTimestepFlag": "false", "dt": "0.01", "nt": "12",
                      "forcing": "isotropicBand", "forcingPower": "0.1", "forcingKf": "2.5"},
    # AB3, adaptive dt, stopped by timeDuration at an iteration that is not a stats
    # iteration (the tail row then keeps the last non-linear/pressure columns)
    "ab3-adaptive-timeDuration": {"velocityTimeStep": "Adams_Bashforth3rdO", "variableTimestepFlag": "true",
                                  "cfl": "0.4", "dt": "0.01", "nt": "1000", "timeDuration": "0.05"},
    # rfForcing: the run ends by writing the shells' ODE state R.N (FluidFlowSimulation.jl:60-62)
    "etd-rf-forcing": {"velocityTimeStep": "ETD3rdO", "variableTimestepFlag": "false", "dt": "0.01", "nt": "10",
                       "forcing": "rfForcing", "TF": "2.0", "alphac": "1.0", "kf": "3.0"},
    # specFil: Stats_fil.txt and the *_fil spectrum files (stats.jl:14-18, 48-52; spec.jl:13-142)
    "etd-specfil-hv": {"velocityTimeStep": "ETD3rdO", "variableTimestepFlag": "false", "dt": "0.01", "nt": "8",
                       "hyperViscosity": "true", "hyperViscosityCoefficient": "1e-5", "specFil": "2"},
    # writeoutput's LES fields (output.jl:22-42): T11..T23, cs, cp and the density's dflux at
    # 5 and 10 (in-loop) and at the tail's 12 (the explicit writeoutput)
    "etd-dynamicsandp-density-les": {"velocityTimeStep": "ETD3rdO", "variableTimestepFlag": "false", "dt": "0.01",
                                     "nt": "12", "lesModel": "dynamicSandP", "sLesModel": "dynamicSmagorinsky",
                                     "densityStratification": "true", "Pr": "1", "densityGradient": "1",
                                     "zAcceleration": "1", "referenceDensity": "1",
                                     "densityLesModel": "vorticityDiffusion"},
    # a run that ends at a multiple of writeTime: the tail's calculate_rhs! writes the final
    # files before the tail's forcing (R, Eh and N of nRfForcing at 5, 10)
    "ab3-nrf-forcing-smagorinsky": {"velocityTimeStep": "Adams_Bashforth3rdO", "variableTimestepFlag": "false",
                                    "dt": "0.01", "nt": "10", "forcing": "nRfForcing", "TF": "2.0",
                                    "alphac": "1.0", "kf": "3.0", "lesModel": "Smagorinsky"},
    # aForcing's R.N is its (nx/2+1) x ny mode matrix
    "etd-a-forcing": {"velocityTimeStep": "ETD3rdO", "variableTimestepFlag": "false", "dt": "0.01", "nt": "11",
                      "forcing": "aForcing", "TF": "2.0", "alphac": "1.0", "kf": "3.0"},
}


@pytest.mark.parametrize("case", sorted(CASES))
def test_run_simulation_files_match_oracle(gpu_pkg, tmp_path, case):
    n = 32
    d = {"nx": str(n), "ny": str(n), "nz": str(n), "xDomainSize": "1.0", "yDomainSize": "1.0",
         "zDomainSize": "1.0", "kinematicViscosity": "0.01", "dtStat": "3", "dtSpec": "4", "writeTime": "5",
         **CASES[case]}
    u = gpu_pkg.random_spectrum(n, k0=3.0, seed=11)
    (tmp_path / "global").write_text("// case\n" + "".join(f"{k} {v}\n" for k, v in d.items()))
    for i in range(3):
        gpu_pkg.write_field(tmp_path / f"u{i + 1}.0", u[i])
    sim = gpu_pkg.run_simulation(tmp_path, precision="FP64")
    ref, outputs, les, forcing = oracle_run(d, u)
    assert sim.iteration == ref.iteration
    sim.close()
    p = Params.from_global(d)
    # Stats.txt, Scales.txt, Numbers.txt
    head, rows = read_rows(tmp_path / "Stats.txt")
    assert head == stats_header(p)
    assert rows[-1, 0] == ref.iteration
    assert rows_err(rows, ref.stats_rows) <= 1e-10
    for name, want in (("Scales.txt", ref.scales_rows), ("Numbers.txt", ref.numbers_rows)):
        _, got = read_rows(tmp_path / name)
        assert rows_err(got, want) <= 1e-10, name
    assert (tmp_path / "Stats_fil.txt").exists() == ("specFil" in d)
    if "specFil" in d:
        head, rows = read_rows(tmp_path / "Stats_fil.txt")
        assert head == stats_header(p)
        assert rows_err(rows, ref.stats_fil_rows) <= 1e-10
    # spectra: every (field, iteration) the oracle recorded is a file with its values
    assert ref.spectra
    for it, sp in ref.spectra.items():
        for key, want in sp.items():
            f = tmp_path / f"{key}.{it}"
            assert f.exists(), f.name
            got = np.loadtxt(f)
            assert got.shape == (len(want), 2)
            scale = max(np.abs(want).max(), 1e-300)
            assert np.allclose(got[:, 1], want, rtol=1e-10, atol=1e-12 * scale), f.name
    # the kz = 0 forcing files of every output (R, Eh = avgK Ef, N; aForcing's R matrix)
    written_f = sorted(f.name for f in tmp_path.glob("*.*") if f.name.split(".")[0] in ("R", "Eh", "N"))
    assert written_f == sorted(f"{k}.{it}" for it, st in forcing.items() for k in st)
    for it, st in forcing.items():
        for k, want in st.items():
            got = np.loadtxt(tmp_path / f"{k}.{it}", ndmin=2 if np.ndim(want) == 2 else 1)
            assert got.shape == np.shape(want), (k, it)
            assert np.allclose(got, want, rtol=1e-10, atol=1e-14 * max(np.abs(want).max(), 1e-300)), (k, it)
    # writeoutput's LES fields: raw Float64 n^3 per field and output iteration
    names = ("T11", "T12", "T13", "T22", "T23", "cs", "cp", "dflux1", "dflux2", "dflux3")
    written_l = sorted(f.name for f in tmp_path.glob("*.*") if f.name.split(".")[0] in names)
    assert written_l == sorted(f"{k}.{it}" for it, st in les.items() for k in st)
    for it, st in les.items():
        for k, want in st.items():
            f = tmp_path / f"{k}.{it}"
            assert f.stat().st_size == 8 * n ** 3
            got = gpu_pkg.read_field(f, n, n, n)
            assert np.linalg.norm(got - want) <= 1e-10 * np.linalg.norm(want), (k, it)
    # field files: exactly the oracle's output iterations, raw Float64 n^3
    written = sorted(int(f.name.split(".")[1]) for f in tmp_path.glob("u1.*") if f.name != "u1.0")
    assert written == sorted(outputs)
    for it, ur in outputs.items():
        for c in range(3):
            f = tmp_path / f"u{c + 1}.{it}"
            assert f.stat().st_size == 8 * n ** 3
            got = gpu_pkg.read_field(f, n, n, n)
            assert np.linalg.norm(got - ur[c]) <= 1e-12 * np.linalg.norm(ur[c]), (it, c)


def test_output_capture_rules(gpu_pkg):
    """ffs_capture_output: output steps are the steps that start at a multiple of writeTime,
    except the first after ffs_initialize (is_output_time, src/simulationtypes.jl:102);
    switched off, no step captures; without an LES model there is nothing to capture."""
    n = 32
    d = {"nx": str(n), "ny": str(n), "nz": str(n), "xDomainSize": "1.0", "yDomainSize": "1.0",
         "zDomainSize": "1.0", "kinematicViscosity": "0.01", "dtStat": "100", "dtSpec": "100", "writeTime": "3",
         "velocityTimeStep": "ETD3rdO", "variableTimestepFlag": "false", "dt": "0.01", "lesModel": "Smagorinsky"}
    u = gpu_pkg.random_spectrum(n, k0=3.0, seed=5)
    sim = gpu_pkg.Simulation.from_global(d, precision="FP64")
    sim.set_fields(*u)
    sim.capture_output(True)
    sim.initialize()
    sim.advance_in_time(1)               # iteration 0: the first step after initialize!
    with pytest.raises(gpu_pkg.FFSError) as e:
        sim.output_fields()
    assert e.value.code == -7
    sim.advance_in_time(3)               # steps 1, 2, 3: the step from 3 captures
    it, f = sim.output_fields()
    assert it == 3 and sorted(f) == ["T11", "T12", "T13", "T22", "T23"]
    sim.capture_output(False)
    sim.advance_in_time(4)               # through 7: the step from 6 does not capture
    assert sim.output_fields()[0] == 3
    sim.close()
    plain = gpu_pkg.Simulation.from_global({k: v for k, v in d.items() if k != "lesModel"}, precision="FP64")
    plain.capture_output(True)
    with pytest.raises(gpu_pkg.FFSError) as e:
        plain.output_fields()
    assert e.value.code == -7
    plain.close()
