"""Known-answer tests that pin the FP64 oracle (the reference itself cannot run here:
no Julia, no FFTW; its only test is a placeholder, test/runtests.jl:5)."""
import math

import numpy as np
import pytest

from oracle.ffs_oracle import ETD3, AB3, Grid, OracleSimulation, Params, fftfreq, rfftfreq, stats_header, taylor_green


def tg_params(n=32, **kw):
    p = Params(nx=n, ny=n, nz=n, nu=0.0333333, integrator="Adams_Bashforth3rdO", variable_dt=False, dt=0.05,
               dt_stat=1, dt_spec=1)
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def test_wavenumbers_match_reference_tables():
    # Globals.jl:95-104
    assert np.array_equal(rfftfreq(8, 1.0), [0, 1, 2, 3, 4])
    assert np.array_equal(fftfreq(8, 1.0), [0, 1, 2, 3, -4, -3, -2, -1])
    assert np.allclose(fftfreq(8, 2.0), [0, 0.5, 1, 1.5, -2, -1.5, -1, -0.5])


@pytest.mark.parametrize("n,mx", [(32, 11), (48, 17), (64, 22), (96, 33), (128, 43), (256, 86)])
def test_dealias_box(n, mx):
    """XRANGE length (Globals.jl:163). For n = 48, 96 the FP64 product (2/3)*(n/2) rounds
    to exactly n/3, so kx = n/3 is kept (k^2 > cutoff^2 is false)."""
    g = Grid(n, n, n)
    assert int(np.argmax(g.dealias[0, 0, :])) == mx
    keep_y = (~g.dealias[0, :, 0]).sum()
    assert keep_y == 2 * mx - 1


def test_taylor_green_initial_stats():
    """E = k = 1/8, <u1^2> = <u2^2> = 1/8, <u3^2> = 0, eps = 3 nu (u1p2 + u2p2) = 0.75 nu."""
    p = tg_params()
    s = OracleSimulation(p, taylor_green(32))
    s.initialize()
    s.advance()
    row = s.stats_rows[0]
    cols = {c: row[i] for i, c in enumerate("iteration,time,u1,u2,u3,u1p2,u2p2,u3p2,kh,kv,kaniso,k,dissh,dissv,diss".split(","))}
    assert cols["u1p2"] == pytest.approx(0.125, rel=1e-13)
    assert cols["u2p2"] == pytest.approx(0.125, rel=1e-13)
    assert abs(cols["u3p2"]) < 1e-28
    assert cols["k"] == pytest.approx(0.125, rel=1e-13)
    assert cols["diss"] == pytest.approx(0.75 * p.nu, rel=1e-13)


def test_projection_divergence_free():
    p = tg_params(n=32)
    rng = np.random.default_rng(0)
    u = [rng.standard_normal((32, 32, 32)) for _ in range(3)]
    s = OracleSimulation(p, u)
    s.initialize()
    s.run(3)
    g = s.g
    div = g.KX * s.u[0] + g.KY * s.u[1] + g.KZ * s.u[2]
    assert np.abs(div).max() < 1e-13 * np.abs(s.u).max()


def test_shear_flow_decays_exactly_under_etd():
    """u = (sin(2z), 0, 0): u x w is a pure gradient, projected away; ETD is exact."""
    n = 32
    z = 2 * np.pi * np.arange(n) / n
    u1 = np.broadcast_to(np.sin(2 * z)[:, None, None], (n, n, n)).copy()
    p = Params(nx=n, ny=n, nz=n, nu=0.05, integrator="ETD3rdO", variable_dt=False, dt=0.1, dt_stat=1000,
               dt_spec=1000)
    s = OracleSimulation(p, (u1, np.zeros_like(u1), np.zeros_like(u1)))
    s.initialize()
    s.run(10)
    ur = s.u_physical()
    expect = u1 * math.exp(-p.nu * 4 * 1.0)
    assert np.abs(ur[0] - expect).max() < 1e-13
    assert np.abs(ur[1]).max() < 1e-13 and np.abs(ur[2]).max() < 1e-13


def test_shear_flow_decays_exactly_under_euler():
    """The same shear flow under Euller (Euller.jl:14-25): u_{n+1} = (1 - nu k^2 dt) u_n with
    the explicit viscous term, so after 10 steps the amplitude is (1 - nu k^2 dt)^10."""
    n = 32
    z = 2 * np.pi * np.arange(n) / n
    u1 = np.broadcast_to(np.sin(2 * z)[:, None, None], (n, n, n)).copy()
    p = Params(nx=n, ny=n, nz=n, nu=0.05, integrator="Euller", variable_dt=False, dt=0.1, dt_stat=1000,
               dt_spec=1000)
    s = OracleSimulation(p, (u1, np.zeros_like(u1), np.zeros_like(u1)))
    s.initialize()
    s.run(10)
    ur = s.u_physical()
    expect = u1 * (1 - p.nu * 4 * 0.1) ** 10
    assert np.abs(ur[0] - expect).max() < 1e-13
    assert np.abs(ur[1]).max() < 1e-13 and np.abs(ur[2]).max() < 1e-13


def test_density_eddy_diffusion_is_a_dissipation():
    """densityLesModel eddyDiffusion (les_real_calc.jl:116-123): the LES flux nu_t grad rho
    with nu_t >= 0 only removes density variance, and rhopr = -sum proj(i k . flux, rho)
    counts it (stats.jl:1032-1053) in trhodiss."""
    n = 32
    rng = np.random.default_rng(3)
    base = {"nx": str(n), "ny": str(n), "nz": str(n), "xDomainSize": "1", "yDomainSize": "1", "zDomainSize": "1",
            "kinematicViscosity": "0.01", "dtStat": "1", "dtSpec": "1000", "writeTime": "1000",
            "velocityTimeStep": "ETD3rdO", "variableTimestepFlag": "false", "dt": "0.005",
            "densityStratification": "true", "Pr": "1", "densityGradient": "0", "zAcceleration": "0",
            "referenceDensity": "1", "lesModel": "Smagorinsky", "densityLesModel": "eddyDiffusion"}
    g = Grid(n, n, n)
    rho = g.real(g.myfourier(rng.standard_normal((n, n, n))) * np.exp(-np.sqrt(g.K2) / 3))
    u = [g.real(g.myfourier(rng.standard_normal((n, n, n))) * np.exp(-np.sqrt(g.K2) / 3)) for _ in range(3)]
    h = stats_header(Params.from_global(base)).split(",")
    s = OracleSimulation(Params.from_global(base), u, rho)
    s.initialize()
    s.run(2)
    rows = np.array(s.stats_rows)
    assert (rows[:, h.index("rhopr")] > 0).all()
    # trhodiss = rhodiss + rhopr (density_stratification_types.jl:52-56)
    assert np.allclose(rows[:, h.index("trhodiss")], rows[:, h.index("rhodiss")] + rows[:, h.index("rhopr")],
                       rtol=1e-14, atol=0)


def test_ab3_coefficients_reduce_to_constant_dt():
    t = AB3(True, 0.1)
    t.dt = t.dt2 = t.dt3 = 0.1
    a, b, c = t.coefficients()
    assert (a, b, c) == pytest.approx((23 * 0.1 / 12, -16 * 0.1 / 12, 5 * 0.1 / 12), rel=1e-14)


def test_etd3_constant_linear_is_exact():
    """With N = 0 every ETD stage is u' = exp(c dt) u."""
    c = -np.linspace(0, 50, 64)
    t = ETD3(False, 0.05, c)
    u = np.ones(64, complex)
    t.initialize(np.zeros(64, complex), 0.05)
    for _ in range(4):
        u = t.step(u, np.zeros(64, complex))
    assert np.allclose(u, np.exp(c * 0.2), rtol=1e-14, atol=0)


def test_etd_phi_taylor_branch_continuity():
    """Coefficients stay continuous across the -c dt = 1e-4 switch (ETD.jl:181-191) up to the
    truncation of the reference's Taylor series (a relative jump below 1e-7)."""
    dt = 0.01
    c = np.array([-1e-2 * (1 - 1e-9), -1e-2 * (1 + 1e-9)])   # straddles -c dt = 1e-4
    t = ETD3(False, dt, c)
    t.set_ABCt()
    for a in (t.At, t.Bt, t.Ct):
        assert abs(a[0] - a[1]) < 1e-7 * abs(a[0])


def test_unforced_energy_budget():
    """dk/dt = -diss + nl + press (nl + press ~ 0: the dealiased transfer conserves energy)."""
    n = 32
    rng = np.random.default_rng(1)
    from oracle.ffs_oracle import Grid as G
    g = G(n, n, n)
    uh = np.stack([g.myfourier(rng.standard_normal((n, n, n))) for _ in range(3)])
    uh = g.project(uh)
    kk = np.sqrt(g.K2)
    uh *= np.exp(-kk / 3)[None]
    u = g.real(uh)
    p = Params(nx=n, ny=n, nz=n, nu=0.02, integrator="ETD3rdO", variable_dt=False, dt=1e-3, dt_stat=1, dt_spec=1000)
    s = OracleSimulation(p, u)
    s.initialize()
    s.run(6)
    rows = np.array(s.stats_rows)
    k = rows[:, 11]
    diss = rows[:, 14]
    nlh, nlv, ph, pv = rows[:, 15], rows[:, 16], rows[:, 17], rows[:, 18]
    assert abs((nlh + nlv)[3]) < 1e-10 * diss[3]
    assert abs((ph + pv)[3]) < 1e-10 * diss[3]
    dkdt = (k[4] - k[2]) / (2 * p.dt)
    assert dkdt == pytest.approx(-diss[3], rel=2e-3)


def test_forcing_injects_epsilon():
    """Isotropic band forcing: power hp + vp = eps (+ O(dt) from the 1/2 |f|^2 term)."""
    n = 32
    rng = np.random.default_rng(2)
    u = [rng.standard_normal((n, n, n)) for _ in range(3)]
    p = Params(nx=n, ny=n, nz=n, nu=0.01, integrator="Adams_Bashforth3rdO", variable_dt=False, dt=1e-4,
               forcing=True, forcing_power=0.1, forcing_kf=2.5, dt_stat=1, dt_spec=1000)
    s = OracleSimulation(p, u)
    s.initialize()
    s.run(2)
    tp = s.stats_rows[-1][-1]
    assert tp == pytest.approx(0.1, rel=1e-3)


def test_reference_cfl_slot_semantics():
    """set_dt! uses max(max|u|, leftover of the last stats reduction) (utils.jl:247-258):
    after a stats step reductionh[1] holds dx_squared_mean(u2) (stats.jl:93)."""
    import copy
    n = 16
    u = taylor_green(n)
    p = Params(nx=n, ny=n, nz=n, nu=0.01, integrator="ETD3rdO", variable_dt=True, cfl=0.5, dt_stat=1,
               dt_spec=1000)
    s = OracleSimulation(p, u)
    s.initialize()
    c = copy.deepcopy(s)
    c.calculate_rhs()
    g = s.g
    expect = float(np.sum(g.w * g.KX ** 2 * np.abs(c.u[1]) ** 2))
    s.advance()
    assert s.slot_u == pytest.approx(expect, rel=1e-12)
    p2 = Params(**{**p.__dict__, "reference_cfl_slot": False})
    s2 = OracleSimulation(p2, u)
    s2.initialize()
    s2.run(2)
    assert s2.slot_u == pytest.approx(s2.umax_hist[-1])


def test_taylor_green_64_ab3_at_its_dt_blows_up():
    """The Taylor-Green 64^3 configuration as written (AB3, nu = 0.0333333, dt = 0.05):
    AB3 treats the viscous term explicitly and nu k_max^2 dt = 0.0333333 * 3 * 21^2 * 0.05
    = 2.2 lies far outside its stability interval, so the energy explodes within 40
    steps. The configuration therefore runs on ETD3 (the reference's default integrator),
    which integrates the viscous term exactly."""
    p = tg_params(n=64, dt_stat=1000, dt_spec=1000)
    s = OracleSimulation(p, taylor_green(64))
    s.initialize()
    e0 = float(np.sum(np.abs(s.u) ** 2))
    for _ in range(40):
        s.advance()
    e = float(np.sum(np.abs(s.u) ** 2))
    assert not (e < 1e6 * e0)      # blown up (or NaN)
    # the same run on ETD3 decays smoothly
    q = tg_params(n=64, integrator="ETD3rdO", dt_stat=1000, dt_spec=1000)
    t = OracleSimulation(q, taylor_green(64))
    t.initialize()
    for _ in range(10):
        t.advance()
    assert 0 < float(np.sum(np.abs(t.u) ** 2)) < e0


def test_config_fixture_is_the_oracle_run():
    """The Taylor-Green 64^3 full-run fixture (tests/golden/configs) starts the way the
    oracle runs now: its first two rows (iterations 0 and 20)."""
    from pathlib import Path
    z = np.load(Path(__file__).resolve().parent / "golden" / "configs" / "tg64_etd3_500.npz")
    d = dict(zip([str(k) for k in z["keys"]], [str(v) for v in z["values"]]))
    s = OracleSimulation(Params.from_global(d), taylor_green(64))
    s.initialize()
    s.run(21)
    assert np.allclose(np.array(s.stats_rows), z["stats"][:2], rtol=1e-12, atol=1e-15)
    assert z["stats"].shape[0] == 26 and z["stats"][-1, 0] == 500


def test_qf_forcing_injects_its_power_split_99_to_1():
    """QfForcing (qfforcing.jl:1-81): the horizontal kz = 0 modes take 0.99 P and the
    (0, 0, kz) modes 0.01 P of the power alveliusP, at every step."""
    d = {"nx": "32", "ny": "32", "nz": "32", "xDomainSize": "1.0", "yDomainSize": "1.0", "zDomainSize": "1.0",
         "kinematicViscosity": "0.01", "dtStat": "1", "dtSpec": "100", "writeTime": "1000",
         "velocityTimeStep": "Adams_Bashforth3rdO", "variableTimestepFlag": "false", "dt": "0.01",
         "forcing": "QfForcing", "alveliusP": "0.25", "alveliusC": "1.0", "alveliusKf": "2.0", "kf": "4.0"}
    rng = np.random.default_rng(3)
    g = Grid(32, 32, 32)
    uh = g.project(np.stack([g.myfourier(rng.standard_normal((32, 32, 32))) for _ in range(3)]))
    s = OracleSimulation(Params.from_global(d), list(g.real(uh * np.exp(-g.K2 / 20)[None])))
    s.initialize()
    s.run(3)
    r = np.array(s.stats_rows)
    assert np.allclose(r[:, -3], 0.99 * 0.25, rtol=1e-12) and np.allclose(r[:, -2], 0.01 * 0.25, rtol=1e-12)
    assert s.stats_rows and stats_header(s.p).endswith("hp,vp,tp")


def test_rf_forcing_shells_match_compute_shells2D():
    """compute_shells2D (utils.jl:161-182) at 32^3: 16 shells, shell 0 is k = 0 alone and
    shell n averages |k_h| over the half plane with round(|k_h|) = n."""
    from oracle.ffs_oracle import PlaneForcing
    p = Params(nx=32, ny=32, nz=32, plane_forcing="rfForcing", pf_tf=1.0, pf_alpha=1.0, pf_kf=3.0)
    f = PlaneForcing(p, Grid(32, 32, 32))
    assert f.nsh == 16 and f.kh[0] == 0.0
    kx, ky = np.arange(17), np.fft.fftfreq(32, 1 / 32)
    K = np.sqrt(kx[None, :] ** 2 + ky[:, None] ** 2)
    for n in (1, 5, 15):
        assert f.kh[n] == pytest.approx(K[np.rint(K) == n].mean(), rel=1e-14)
    assert np.array_equal(f.Zf, (f.kh <= 3.0).astype(np.float64)) and f.Zf[2] == 1.0 and f.Zf[4] == 0.0
