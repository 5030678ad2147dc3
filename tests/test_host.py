"""Host logic on CPU: the C ABI library loads and exports what include/ffs.h declares,
the `global` parser and parameter mapping, file formats and initial conditions."""
import ctypes
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


def header_functions():
    src = (ROOT / "include" / "ffs.h").read_text()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(ffs_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol(pkg):
    import __graft_entry__ as ge
    if not pkg.lib_available():
        ge.build()
    L = pkg.load()
    names = header_functions()
    assert set(names) == set(pkg.EXPORTS)
    for n in names:
        assert hasattr(L, n), n


def test_julia_binding_calls_only_declared_symbols():
    """Every entry point the Julia ccall shim binds is declared in include/ffs.h (the shim
    cannot run here: no Julia in the image)."""
    src = (ROOT / "fluidflowsimulation.jl_gb300" / "julia" / "FFSEngine.jl").read_text()
    called = set(re.findall(r"ccall\(\(:(ffs_[a-z0-9_]+)", src))
    assert called, "no ccall found"
    assert called <= set(header_functions()), sorted(called - set(header_functions()))


def test_julia_params_struct_matches_header():
    """The Julia FFSParams mirrors ffs_params field by field (names, order, C types)."""
    h = re.sub(r"/\*.*?\*/", "", (ROOT / "include" / "ffs.h").read_text(), flags=re.S)
    body = re.search(r"typedef struct ffs_params \{(.*?)\} ffs_params;", h, flags=re.S).group(1)
    cfields = []
    for decl in body.split(";"):
        m = re.match(r"\s*(int32_t|int64_t|double)\s+(.+)", decl.strip())
        if m:
            cfields += [(n.strip(), m.group(1)) for n in m.group(2).split(",")]
    jl = (ROOT / "fluidflowsimulation.jl_gb300" / "julia" / "FFSEngine.jl").read_text()
    jbody = re.search(r"mutable struct FFSParams(.*?)FFSParams\(\) = new\(\)", jl, flags=re.S).group(1)
    jmap = {"Int32": "int32_t", "Int64": "int64_t", "Float64": "double"}
    jfields = [(n, jmap[t]) for n, t in re.findall(r"(\w+)::(\w+)", jbody)]
    assert jfields == cfields


def test_params_default_matches_reference_defaults(pkg):
    p = pkg.FFSParams()
    assert pkg.load().ffs_params_default(ctypes.byref(p)) == 0
    assert p.cutoff == pytest.approx(2 / 3)          # Globals.jl:132
    assert p.cfl == pytest.approx(0.18)              # simulationtypes.jl:310
    assert p.integrator == pkg.FFS_ETD3              # simulationtypes.jl:308
    assert p.variable_dt == 1                        # simulationtypes.jl:309
    assert p.hv_m == 2 and p.smag_c == pytest.approx(0.17)


def test_create_without_gpu_fails_cleanly(pkg):
    """Without a GPU, ffs_create returns an error code and a message instead of crashing.
    Runs in a child process: a failed CUDA driver load leaves the process in an odd state."""
    import subprocess
    import sys
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    code = (
        "import sys, ctypes; sys.path.insert(0, %r)\n"
        "import __graft_entry__ as ge\n"
        "pkg = ge.load_package(); L = pkg.load(); p = pkg.FFSParams(); L.ffs_params_default(ctypes.byref(p))\n"
        "h = ctypes.c_void_p(); rc = L.ffs_create(ctypes.byref(p), ctypes.byref(h))\n"
        "print(rc, L.ffs_last_error(None).decode())\n"
    ) % str(ROOT)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    rc, msg = r.stdout.strip().split(" ", 1)
    assert int(rc) < 0 and msg


def test_readglobal_and_parameters(pkg, tmp_path):
    (tmp_path / "global").write_text("""// comment
kinematicViscosity 0.03333333
xDomainSize 1.0
yDomainSize 1.0
zDomainSize 2π

nx 64
ny 64
nz 64
nt 500
dt 0.05
dtStat 20
dtSpec 20
writeTime 100
velocityTimeStep Adams_Bashforth3rdO
variableTimestepFlag false
hyperViscosity true
hyperViscosityCoefficient 1e-12
forcing isotropicBand
forcingPower 0.1
forcingKf 2.5
precision FP32
""")
    d = pkg.readglobal(tmp_path / "global")
    assert d["zDomainSize"] == "2π" and d["nt"] == "500"
    p = pkg.parameters(d)
    assert (p.nx, p.ny, p.nz) == (64, 64, 64)
    assert p.lz == pytest.approx(2 * np.pi)
    assert p.integrator == pkg.FFS_AB3 and p.variable_dt == 0 and p.dt == pytest.approx(0.05)
    assert p.hyperviscosity == 1 and p.hv_nu == pytest.approx(1e-12) and p.hv_m == 2
    assert p.forcing == 1 and p.precision == pkg.FFS_FP32
    assert p.dt_stat == 20 and p.dt_spec == 20 and p.write_time == 100


def test_parameters_requires_dtspec(pkg):
    """The reference raises KeyError without dtSpec (simulationtypes.jl:262)."""
    d = {"nx": "8", "ny": "8", "nz": "8", "xDomainSize": "1", "yDomainSize": "1", "zDomainSize": "1",
         "kinematicViscosity": "0.1", "dtStat": "1", "writeTime": "1"}
    with pytest.raises(KeyError):
        pkg.parameters(d)


def test_parameters_rejects_out_of_scope_models(pkg):
    d = {"nx": "8", "ny": "8", "nz": "8", "xDomainSize": "1", "yDomainSize": "1", "zDomainSize": "1",
         "kinematicViscosity": "0.1", "dtStat": "1", "dtSpec": "1", "writeTime": "1",
         "lesModel": "fakeSmagorinsky"}
    with pytest.raises(ValueError):
        pkg.parameters(d)
    for m in ("dynamicSandP", "piomelliSandP"):
        with pytest.raises(ValueError):
            pkg.parameters(dict(d, lesModel=m, sLesModel="Smagorinsky"))
    with pytest.raises(ValueError):
        pkg.parameters(dict(d, lesModel="SandP", sLesModel="Silvis"))
    p = pkg.parameters(dict(d, lesModel="SandP", sLesModel="dynamicSmagorinsky"))   # les_types.jl:401-416
    assert (p.les_model, p.sandp_cb, p.les_dynp) == (5, 0.09, 0)


def test_parameters_les_models(pkg):
    """lesModel keys and defaults of les_types (les_types.jl:360-395), the same in the
    oracle's Params."""
    import math
    from oracle.ffs_oracle import Params
    base = {"nx": "32", "ny": "32", "nz": "32", "xDomainSize": "1", "yDomainSize": "1", "zDomainSize": "1",
            "kinematicViscosity": "0.1", "dtStat": "1", "dtSpec": "1", "writeTime": "1"}
    dx = 2 * math.pi / 32 / (2 / 3)
    cases = {  # lesModel keys -> (model id, constant, cp, cb, filter width passed to the engine)
        ("Vreman",): (1, 0.032, None, 0.0, 0.0),
        ("productionViscosity",): (2, 0.4, None, 0.0, 0.0),
        ("Silvis",): (3, math.sqrt(0.17), 5.0, 0.0, 0.0),
        ("stableNonLinear",): (4, 0.1, None, 0.0, 0.0),
        ("SandP", "Smagorinsky"): (0, 0.17, None, 0.09, 2 * dx),
        ("SandP", "productionViscosity"): (2, 0.1, None, 0.09, 0.0),
    }
    for keys, (mid, c, cp, cb, fw) in cases.items():
        d = dict(base, lesModel=keys[0])
        if len(keys) > 1:
            d["sLesModel"] = keys[1]
        p = pkg.parameters(d)
        assert (p.les, p.les_model, p.sandp_cb) == (1, mid, cb), keys
        assert p.smag_c == pytest.approx(c) and p.filter_width == pytest.approx(fw)
        if cp is not None:
            assert p.les_cp == cp
        o = Params.from_global(d)
        assert o.les and o.smag_c == pytest.approx(c) and o.sandp_cb == cb
        assert o.filter_width == pytest.approx(fw if fw else dx)
    # dynamicSmagorinsky (les_types.jl:388-392): test filter twice the filter width unless
    # TestFilterWidth is given, cmin default 0
    p = pkg.parameters(dict(base, lesModel="dynamicSmagorinsky"))
    assert (p.les, p.les_model, p.filter_width, p.les_test_width, p.les_cmin) == (1, 5, 0.0, 0.0, 0.0)
    o = Params.from_global(dict(base, lesModel="dynamicSmagorinsky"))
    assert (o.les_model, o.les_cmin) == ("dynamicSmagorinsky", 0.0)
    assert o.filter_width == pytest.approx(dx) and o.les_test_width == pytest.approx(2 * dx)
    p = pkg.parameters(dict(base, lesModel="piomelliSmagorinsky"))
    assert (p.les, p.les_model, p.les_test_width) == (1, 6, 0.0)
    for m, dp in (("dynamicSandP", 1), ("piomelliSandP", 2)):   # les_types.jl:426-455
        for sm, mid in (("dynamicSmagorinsky", 5), ("piomelliSmagorinsky", 6)):
            p = pkg.parameters(dict(base, lesModel=m, sLesModel=sm))
            assert (p.les, p.les_model, p.les_dynp) == (1, mid, dp)
            o = Params.from_global(dict(base, lesModel=m, sLesModel=sm))
            assert (o.les_model, o.les_dynp) == (sm, m)
    d = dict(base, lesModel="dynamicSmagorinsky", filterWidth="0.2", TestFilterWidth="0.5", cmin="-0.1")
    p, o = pkg.parameters(d), Params.from_global(d)
    assert (p.filter_width, p.les_test_width, p.les_cmin) == (0.2, 0.5, -0.1)
    assert (o.filter_width, o.les_test_width, o.les_cmin) == (0.2, 0.5, -0.1)


def test_parameters_hyperviscosity_kinds(pkg):
    """hyperViscosity spectralBarrier (simulationtypes.jl:294-297) and densityHyperViscosity
    (density_stratification_types.jl:137-148), the same in the oracle's Params."""
    import math
    from oracle.ffs_oracle import Params
    base = {"nx": "48", "ny": "48", "nz": "48", "xDomainSize": "1", "yDomainSize": "1", "zDomainSize": "1",
            "kinematicViscosity": "0.1", "dtStat": "1", "dtSpec": "1", "writeTime": "1"}
    d = dict(base, hyperViscosity="spectralBarrier")
    p, o = pkg.parameters(d), Params.from_global(d)
    assert (p.hyperviscosity, p.hv_kind, p.hv_initk, p.hv_endk) == (1, 1, 0.0, 0.0)   # engine defaults
    assert o.hv_kind == "barrier"
    assert o.hv_initk == pytest.approx((2 / 3) * 2 * 24 / 3) and o.hv_endk == pytest.approx(math.sqrt(2) * 24)
    d = dict(base, hyperViscosity="spectralBarrier", initk="3", endk="9.5")
    assert (pkg.parameters(d).hv_initk, pkg.parameters(d).hv_endk) == (3.0, 9.5)
    dens = dict(base, densityStratification="true", Pr="1", densityGradient="1", zAcceleration="1",
                referenceDensity="1")
    d = dict(dens, densityHyperViscosity="true", densityHyperViscosityCoefficient="1e-6", densityHyperViscosityM="3")
    p, o = pkg.parameters(d), Params.from_global(d)
    assert (p.rho_hv, p.rho_hv_nu, p.rho_hv_m) == (1, 1e-6, 3) and (o.rho_hv, o.rho_hv_m) == ("power", 3)
    d = dict(dens, densityHyperViscosity="spectralBarrier", densityEndk="20")
    p, o = pkg.parameters(d), Params.from_global(d)
    assert (p.rho_hv, p.rho_hv_endk) == (2, 20.0) and (o.rho_hv, o.rho_hv_endk) == ("barrier", 20.0)


def test_parameters_integrators(pkg):
    """velocityTimeStep (simulationtypes.jl:308-318): ETD3rdO (default), Adams_Bashforth3rdO,
    Euller; the oracle's explicit flag covers both explicit integrators."""
    from oracle.ffs_oracle import Params
    base = {"nx": "16", "ny": "16", "nz": "16", "xDomainSize": "1", "yDomainSize": "1", "zDomainSize": "1",
            "kinematicViscosity": "0.1", "dtStat": "1", "dtSpec": "1", "writeTime": "1"}
    for name, code, explicit in (("ETD3rdO", 0, False), ("Adams_Bashforth3rdO", 1, True), ("Euller", 2, True)):
        d = dict(base, velocityTimeStep=name)
        assert pkg.parameters(d).integrator == code
        assert Params.from_global(d).ab3 == explicit
    assert pkg.parameters(base).integrator == 0
    with pytest.raises(ValueError):
        pkg.parameters(dict(base, velocityTimeStep="RK4"))


def test_parameters_density_and_scalar_les(pkg):
    """densityLesModel (density_stratification_types.jl:176-185) and the passive scalar's LES
    diffusion under lesModel (simulationtypes.jl:334-346): eddy diffusion by default,
    vorticity diffusion with its coefficient (0.1 for the density, 1.0 for the scalar)."""
    from oracle.ffs_oracle import Params
    base = {"nx": "32", "ny": "32", "nz": "32", "xDomainSize": "1", "yDomainSize": "1", "zDomainSize": "1",
            "kinematicViscosity": "0.1", "dtStat": "1", "dtSpec": "1", "writeTime": "1"}
    dens = dict(base, densityStratification="true", Pr="1", densityGradient="1", zAcceleration="1",
                referenceDensity="1", lesModel="Smagorinsky")
    scal = dict(base, passiveScalar="true", scalarPr="1", scalarGradient="1", lesModel="Vreman")
    cases = [
        (dict(dens), 0, 0.0, ""),
        (dict(dens, densityLesModel="eddyDiffusion"), 1, 0.0, "eddy"),
        (dict(dens, densityLesModel="vorticityDiffusion"), 2, 0.1, "vorticity"),
        (dict(dens, densityLesModel="vorticityDiffusion", densityVorticityCoefficient="0.25"), 2, 0.25, "vorticity"),
        (dict(scal), 1, 0.0, "eddy"),
        (dict(scal, scalarLesModel="vorticityDiffusion"), 2, 1.0, "vorticity"),
        (dict(scal, scalarLesModel="vorticityDiffusion", scalarVorticityCoefficient="0.5"), 2, 0.5, "vorticity"),
        (dict(base, passiveScalar="true", scalarPr="1", scalarGradient="1", scalarLesModel="vorticityDiffusion"),
         0, 0.0, ""),
    ]
    for d, kind, c, okind in cases:
        p, o = pkg.parameters(d), Params.from_global(d)
        assert (p.rho_les, p.rho_les_c) == (kind, c), d
        assert (o.rho_les, o.rho_les_c) == (okind, c), d
    # without lesModel the reference's density flux keeps a bare grad rho: refused
    d = dict(dens, densityLesModel="eddyDiffusion")
    del d["lesModel"]
    with pytest.raises(ValueError):
        pkg.parameters(d)
    with pytest.raises(ValueError):
        Params.from_global(d)


def test_write_dlm_matches_julia_writedlm(pkg, tmp_path):
    """writedlm's default layout (the R.N, Eh.N and N.N files): one value per line for a
    vector, tab-separated for an iterator of pairs or a matrix's rows, values as Julia
    prints them."""
    pkg.write_dlm(tmp_path / "v", [0.5, 2.0, 1e-5])
    assert (tmp_path / "v").read_text() == "0.5\n2.0\n1.0e-5\n"
    pkg.write_dlm(tmp_path / "p", np.stack([[1.0, 2.0], [0.25, 3.0]], 1))
    assert (tmp_path / "p").read_text() == "1.0\t0.25\n2.0\t3.0\n"
    pkg.write_dlm(tmp_path / "m", np.array([[1.0, 0.0, 2.5], [0.0, 4.0, 0.0]]))
    assert (tmp_path / "m").read_text() == "1.0\t0.0\t2.5\n0.0\t4.0\t0.0\n"


def test_parse_number(pkg):
    assert pkg.parse_number("2π") == pytest.approx(2 * np.pi)
    assert pkg.parse_number("2pi/128") == pytest.approx(2 * np.pi / 128)
    assert pkg.parse_number("1e-3") == 1e-3
    with pytest.raises(ValueError):
        pkg.parse_number("__import__('os')")


def test_julia_float_formatting(pkg):
    assert pkg.julia_float(0.125) == "0.125"
    assert pkg.julia_float(1.0) == "1.0"
    assert pkg.julia_float(1e-5) == "1.0e-5"
    assert pkg.julia_float(2.5e-20) == "2.5e-20"
    assert pkg.stats_line([20.0, 1.0, 0.5]) == "20,1.0,0.5\n"


def test_field_file_roundtrip(pkg, tmp_path):
    a = np.random.default_rng(0).standard_normal((4, 6, 8))
    pkg.write_field(tmp_path / "u1.0", a)
    assert (tmp_path / "u1.0").stat().st_size == 8 * a.size
    b = pkg.read_field(tmp_path / "u1.0", 8, 6, 4)
    assert np.array_equal(a, b)
    pad = np.zeros((4, 6, 10))
    pad[:, :, :8] = a
    pad.astype("<f8").tofile(str(tmp_path / "u2.0"))
    assert np.array_equal(pkg.read_field(tmp_path / "u2.0", 8, 6, 4), a)


def test_random_spectrum_properties(pkg):
    u = pkg.random_spectrum(32, k0=4.0, seed=3)
    urms = np.sqrt(np.mean(u[0] ** 2 + u[1] ** 2 + u[2] ** 2) / 3)
    assert urms == pytest.approx(1.0, rel=1e-12)
    uh = [np.fft.rfftn(x) for x in u]
    k = np.fft.fftfreq(32, 1 / 32)
    kx = np.arange(17)
    div = kx[None, None, :] * uh[0] + k[None, :, None] * uh[1] + k[:, None, None] * uh[2]
    assert np.abs(div).max() < 1e-10 * np.abs(uh[0]).max()
    # reproducible for a seed, different for another
    assert np.array_equal(u[0], pkg.random_spectrum(32, k0=4.0, seed=3)[0])
    assert not np.array_equal(u[0], pkg.random_spectrum(32, k0=4.0, seed=4)[0])
    # dealiased: nothing beyond |k| = n/3 on each axis
    assert np.abs(uh[0][:, :, 11:]).max() < 1e-10


def test_taylor_green_matches_readme(pkg):
    u1, u2, u3 = pkg.taylor_green(16)
    x = 2 * np.pi * 3 / 16
    y = 2 * np.pi * 5 / 16
    z = 2 * np.pi * 7 / 16
    assert u1[7, 5, 3] == pytest.approx(np.cos(x) * np.sin(y) * np.sin(z))
    assert u2[7, 5, 3] == pytest.approx(-np.sin(x) * np.cos(y) * np.sin(z))
    assert not u3.any()


def test_bench_byte_models():
    """The roofline byte models of bench.py: the 69A effective-bandwidth convention per
    pass adds up to the step, and the retained-mode minimum counts the pruned sizes
    C = Mx NYR NZR, V = Mx NYR n, U = Mx n^2 (256^3: Mx = 86, NYR = NZR = 171)."""
    import sys
    sys.path.insert(0, str(ROOT))
    import bench
    n, elem = 256, 8
    m = bench.model_bytes(n, elem)
    A = (n // 2 + 1) * n * n * elem
    assert m["step"] == 69 * A
    assert sum(v for k, v in m.items() if k != "step") == m["step"]
    r = bench.algorithmic_bytes(n, elem)
    C, V, U = 86 * 171 * 171 * elem, 86 * 171 * n * elem, 86 * n * n * elem
    assert r["inv_z"] == 3 * C + 6 * V and r["x_pass"] == 9 * U and r["update"] == 18 * C
    assert r["step"] == 24 * C + 18 * V + 18 * U
    f = bench.algorithmic_flops(n)
    assert f["x_pass"] == 9 * n * n * 2.5 * n * 8
    assert f["inv_z"] == 6 * 86 * 171 * 5 * n * 8
    assert sum(v for k, v in f.items() if k != "step") == f["step"]


def test_gpu_parity_cases_parse_on_both_sides(pkg):
    """Every global of the GPU parity cases parses in the host mirror and in the oracle,
    with the same integrator, LES model, fourth field and forcing (a parse regression
    shows here without a GPU)."""
    import sys
    from pathlib import Path
    from oracle.ffs_oracle import Params
    sys.path.insert(0, str(Path(__file__).resolve().parent))
    from test_gpu_parity import FIXED_CASES, SPEC_CASES
    integ = {"ETD3rdO": 0, "Adams_Bashforth3rdO": 1, "Euller": 2}
    for name, d in list(FIXED_CASES.items()) + list(SPEC_CASES.items()):
        p, o = pkg.parameters(d), Params.from_global(d)
        assert p.integrator == integ[o.integrator], name
        assert bool(p.les) == o.les and bool(p.density) == o.density and bool(p.passive_scalar) == o.scalar, name
        assert p.rho_les == {"": 0, "eddy": 1, "vorticity": 2}[o.rho_les], name
        assert bool(p.plane_forcing) == bool(o.plane_forcing) and bool(p.forcing) == o.forcing, name
        assert (p.spec_fil != 0) == (o.spec_fil != 0) and bool(p.hyperviscosity) == o.hv, name
