"""Batched serving (ffs_server_*) on the GPU.

- A request's results are the same alone and in a mix of uneven grids and models
  (batch invariance): fields bit-identical, stats rows to 1e-12 relative.
- The batched step computes what the single-simulation step computes (FP32, the same
  generic x pass): fields and stats to 1e-6 relative.
- FP32 batched results are within 1e-4 of the FP64 oracle after 10 steps.
- Admission respects the memory budget; unsupported requests fail at submit.
"""
import numpy as np
import pytest

from oracle.ffs_oracle import OracleSimulation, Params

pytestmark = pytest.mark.gpu


def gdict(n, les=False, integ="Adams_Bashforth3rdO", adaptive=True, nu="0.005", dtstat=4):
    d = {"nx": str(n), "ny": str(n), "nz": str(n), "xDomainSize": "1.0", "yDomainSize": "1.0",
         "zDomainSize": "1.0", "kinematicViscosity": nu, "dtStat": str(dtstat), "dtSpec": "100000",
         "writeTime": "100000", "velocityTimeStep": integ, "variableTimestepFlag": "true" if adaptive else "false",
         "cfl": "0.5", "dt": "0.002"}
    if les:
        d.update({"lesModel": "Smagorinsky", "smagorinskyConstant": "0.17"})
    return d


MIX = [  # (n, les, integrator, adaptive, nt, seed)
    (32, False, "Adams_Bashforth3rdO", True, 12, 1),
    (48, True, "Adams_Bashforth3rdO", True, 9, 2),
    (64, False, "ETD3rdO", False, 7, 3),
    (96, True, "ETD3rdO", False, 5, 4),
    (32, True, "Adams_Bashforth3rdO", True, 15, 5),
    (64, False, "Adams_Bashforth3rdO", True, 10, 6),
    (128, True, "Adams_Bashforth3rdO", True, 6, 7),
    (128, False, "Adams_Bashforth3rdO", True, 8, 8),
]


def fields_of(pkg, case):
    return pkg.random_spectrum(case[0], k0=3.0, seed=case[5])


def submit_case(srv, case, u):
    n, les, integ, adaptive, nt, seed = case
    return srv.submit(gdict(n, les, integ, adaptive), u, nt, keep_fields=True)


def test_batch_invariance(gpu_pkg):
    us = [fields_of(gpu_pkg, c) for c in MIX]
    with gpu_pkg.Server(max_active=16) as srv:
        srv.pause()   # queue the whole mix, then admit it at once
        ids = [submit_case(srv, c, u) for c, u in zip(MIX, us)]
        srv.pause(False)
        mixed = []
        for rid in ids:
            r = srv.wait(rid, timeout=600)
            assert r["status"] == 0
            mixed.append((srv.fields(rid), srv.stats_rows(rid), r))
        assert srv.info()["peak_active"] == len(MIX)
    for case, u, (fm, sm, rm) in zip(MIX, us, mixed):
        with gpu_pkg.Server(max_active=4) as srv:
            rid = submit_case(srv, case, u)
            r = srv.wait(rid, timeout=600)
            fa, sa = srv.fields(rid), srv.stats_rows(rid)
        assert r["iteration"] == rm["iteration"] == case[4]
        assert r["time"] == rm["time"]
        for c in range(3):
            assert np.array_equal(fa[c], fm[c]), (case, c)
        assert sa.shape == sm.shape and sa.shape[0] >= 2
        assert np.allclose(sa, sm, rtol=1e-12, atol=1e-12 * np.abs(sm).max()), case


@pytest.mark.parametrize("case", [MIX[1], MIX[2], MIX[3], MIX[6], MIX[7]])
def test_batched_step_matches_single_engine(gpu_pkg, case):
    n, les, integ, adaptive, nt, seed = case
    d = gdict(n, les, integ, adaptive)
    u = gpu_pkg.random_spectrum(n, k0=3.0, seed=seed)
    with gpu_pkg.Server() as srv:
        rid = srv.submit(d, u, nt, keep_fields=True)
        r = srv.wait(rid, timeout=600)
        fb, sb = srv.fields(rid), srv.stats_rows(rid)
    p = gpu_pkg.parameters(d, precision="FP32")
    p.kernel_variant = 1
    sim = gpu_pkg.Simulation(p)
    sim.set_fields(*u)
    sim.initialize()
    sim.advance_in_time(nt)
    fs, ss = sim.fields(), sim.records()
    assert sim.iteration == r["iteration"]
    for c in range(3):
        assert np.linalg.norm(fb[c] - fs[c]) <= 1e-6 * np.linalg.norm(fs[c])
    assert sb.shape == ss.shape
    assert np.allclose(sb, ss, rtol=1e-6, atol=1e-6 * np.abs(ss).max())
    sim.close()


def test_batched_fp32_against_oracle(gpu_pkg):
    d = gdict(32, adaptive=False, nu="0.01", dtstat=2)
    d["dt"] = "0.01"
    u = gpu_pkg.random_spectrum(32, k0=3.0, seed=7)
    with gpu_pkg.Server() as srv:
        rid = srv.submit(d, u, 10, keep_fields=True)
        srv.wait(rid, timeout=600)
        f = srv.fields(rid)
    ref = OracleSimulation(Params.from_global(d), u)
    ref.initialize()
    ref.run(10)
    g = ref.g
    for c in range(3):
        uh = g.myfourier(f[c])
        assert np.linalg.norm(uh - ref.u[c]) <= 1e-4 * np.linalg.norm(ref.u[c]), c


def test_admission_respects_memory_budget(gpu_pkg):
    pkg = gpu_pkg
    d = gdict(64)
    u = pkg.random_spectrum(64, k0=3.0, seed=9)
    # one 64^3 simulation's buffers, measured through the single-simulation path
    sim = pkg.Simulation(pkg.parameters(d, precision="FP32"))
    one = sim.device_bytes
    sim.close()
    budget = int(2.2 * one)   # two simulations fit, a third does not
    with pkg.Server(memory_budget=budget, max_active=8) as srv:
        ids = [srv.submit(d, u, 20) for _ in range(5)]
        for rid in ids:
            assert srv.wait(rid, timeout=600)["status"] == 0
        info = srv.info()
    assert info["peak_active"] <= 2
    assert info["peak_bytes"] <= budget
    assert info["sim_steps"] == 5 * 20


def test_zero_steps_and_errors(gpu_pkg):
    pkg = gpu_pkg
    d = gdict(32)
    u = pkg.random_spectrum(32, k0=3.0, seed=4)
    with pkg.Server() as srv:
        rid = srv.submit(d, u, 0, keep_fields=True)
        r = srv.wait(rid, timeout=600)
        assert r["status"] == 0 and r["iteration"] == 0
        f = srv.fields(rid)
        for c in range(3):   # the dealiased initial field
            assert np.linalg.norm(f[c] - u[c]) <= 1e-2 * np.linalg.norm(u[c])
        with pytest.raises(pkg.FFSError):
            srv.submit(gdict(256), [np.zeros((256, 256, 256))] * 3, 1)
        p64 = pkg.parameters(d, precision="FP64")
        with pytest.raises(pkg.FFSError):
            srv.submit(p64, u, 1)
        rid2 = srv.submit(d, u, 50)
        with pytest.raises(pkg.FFSError):
            srv.fields(rid2)   # not finished (or finished without keep_fields)
        srv.wait(rid2, timeout=600)
        srv.release(rid2)
        with pytest.raises(pkg.FFSError):
            srv.poll(rid2)


def test_engines_of_different_sizes_coexist(gpu_pkg):
    """A small engine created after a large one must not break the large one (the
    per-kernel shared-memory limit is process-wide)."""
    pkg = gpu_pkg
    big = pkg.Simulation.from_global(gdict(128, les=True), precision="FP32")
    big.set_fields(*pkg.random_spectrum(128, k0=3.0, seed=1))
    big.initialize()
    small = pkg.Simulation.from_global(gdict(32, les=True), precision="FP32")
    small.set_fields(*pkg.random_spectrum(32, k0=3.0, seed=2))
    small.initialize()
    small.advance_in_time(2)
    big.advance_in_time(2)
    assert big.iteration == 2 and small.iteration == 2
    big.close()
    small.close()


def _wait_until(pred, timeout=120.0):
    import time
    t0 = time.perf_counter()
    while not pred():
        assert time.perf_counter() - t0 < timeout, "condition not reached in time"
        time.sleep(0.002)


def _alone(pkg, case, u):
    with pkg.Server(max_active=4) as srv:
        rid = submit_case(srv, case, u)
        r = srv.wait(rid, timeout=600)
        return srv.fields(rid), srv.stats_rows(rid), r


STAGGERED = [  # (n, les, integrator, adaptive, nt, seed): the first runs long, the others join it
    (64, False, "Adams_Bashforth3rdO", True, 400, 21),
    (32, True, "Adams_Bashforth3rdO", True, 120, 22),
    (128, False, "Adams_Bashforth3rdO", True, 40, 23),
    (48, True, "ETD3rdO", False, 60, 24),
]


def test_continuous_batching_requests_join_a_running_batch(gpu_pkg):
    """Requests submitted while others are on the GPU (no pause: each is submitted only
    after the batch has taken steps with the earlier ones) are admitted into the running
    batch, overlap with it, and give bit-identical fields (stats rows to 1e-12) to the
    same request run alone."""
    pkg = gpu_pkg
    us = [fields_of(pkg, c) for c in STAGGERED]
    with pkg.Server(max_active=8) as srv:
        ids = [submit_case(srv, STAGGERED[0], us[0])]
        for case, u in zip(STAGGERED[1:], us[1:]):
            prev = ids[-1]
            _wait_until(lambda: srv.poll(prev)["state"] == "running")
            steps = srv.info()["batch_steps"]
            _wait_until(lambda: srv.info()["batch_steps"] >= steps + 10)
            ids.append(submit_case(srv, case, u))
        res = [srv.wait(rid, timeout=600) for rid in ids]
        mixed = [(srv.fields(rid), srv.stats_rows(rid)) for rid in ids]
        info = srv.info()
    # each later request was admitted while the first one was still running
    first = res[0]
    for r in res[1:]:
        assert first["admit_s"] < r["admit_s"] < first["done_s"]
    assert info["peak_active"] >= 2
    for case, u, (fm, sm), rm in zip(STAGGERED, us, mixed, res):
        fa, sa, ra = _alone(pkg, case, u)
        assert ra["iteration"] == rm["iteration"] == case[4]
        for c in range(3):
            assert np.array_equal(fa[c], fm[c]), (case, c)
        assert sa.shape == sm.shape
        assert np.allclose(sa, sm, rtol=1e-12, atol=1e-12 * np.abs(sm).max()), case


def test_diverged_request_leaves_the_batch_early(gpu_pkg):
    """A request whose initial field holds a NaN (injected on the host) is retired with
    FFS_ENAN within a few health intervals, long before its nt, and frees its slot; the
    requests beside it finish unchanged (bit-identical to alone)."""
    pkg = gpu_pkg
    good = [(64, False, "Adams_Bashforth3rdO", True, 150, 31), (48, True, "Adams_Bashforth3rdO", True, 100, 32)]
    us = [fields_of(pkg, c) for c in good]
    bad_case = (32, False, "Adams_Bashforth3rdO", True, 5000, 33)
    ub = [x.copy() for x in fields_of(pkg, bad_case)]
    ub[1][5, 6, 7] = np.nan
    with pkg.Server(max_active=3) as srv:
        srv.pause()
        ids = [submit_case(srv, c, u) for c, u in zip(good, us)]
        bad = submit_case(srv, bad_case, ub)
        srv.pause(False)
        with pytest.raises(pkg.FFSError) as e:
            srv.wait(bad, timeout=600)
        assert e.value.code == -4
        rb = srv.poll(bad)
        assert rb["status"] == -4
        assert 0 < rb["iteration"] <= 64          # retired after a few health intervals
        # its slot is free again: a further request is admitted and finishes
        extra = submit_case(srv, good[1], us[1])
        res = [srv.wait(rid, timeout=600) for rid in ids + [extra]]
        mixed = [srv.fields(rid) for rid in ids + [extra]]
    assert all(r["status"] == 0 for r in res)
    for case, u, fm in zip(good + [good[1]], us + [us[1]], mixed):
        fa, _, _ = _alone(pkg, case, u)
        for c in range(3):
            assert np.array_equal(fa[c], fm[c]), (case, c)


def test_cancel_queued_and_running_requests(gpu_pkg):
    pkg = gpu_pkg
    long_case = (64, False, "Adams_Bashforth3rdO", True, 200000, 41)
    short_case = (32, False, "Adams_Bashforth3rdO", True, 20, 42)
    ul, us_ = fields_of(pkg, long_case), fields_of(pkg, short_case)
    with pkg.Server(max_active=1) as srv:
        a = submit_case(srv, long_case, ul)
        _wait_until(lambda: srv.poll(a)["state"] == "running")
        b = submit_case(srv, short_case, us_)          # waits: one slot, held by a
        assert srv.poll(b)["state"] == "queued"
        srv.cancel(b)
        _wait_until(lambda: srv.poll(b)["status"] == -8, timeout=30)
        steps = srv.info()["batch_steps"]
        _wait_until(lambda: srv.info()["batch_steps"] >= steps + 5)
        srv.cancel(a)
        with pytest.raises(pkg.FFSError) as e:
            srv.wait(a, timeout=600)
        assert e.value.code == -8
        ra = srv.poll(a)
        assert 0 < ra["iteration"] < long_case[4]
        assert srv.stats_rows(a).shape[0] >= 1        # the records of the steps it took
        c = submit_case(srv, short_case, us_)          # the slot is free again
        assert srv.wait(c, timeout=600)["status"] == 0
        with pytest.raises(pkg.FFSError):
            srv.cancel(c)                              # already finished


# The size classes' kernel forms (ffs_server_cfg.class_forms / autotune): every form of
# every pass computes the same step. Forms 1 and 2 force the one-line-per-thread y/z
# kernels (8 and 4 kx lines a tile) and the generic x passes (4 and 2 lines) on every
# class; the autotuned server keeps the fastest form per pass. Each result is compared
# with the default forms' (FP32 rounding: 1e-5) and with the FP64 oracle (1e-4).
FORM_MIX = [MIX[0], MIX[1], MIX[2], MIX[3], MIX[6], MIX[7]]


def _run_mix(pkg, mix, **kw):
    us = [fields_of(pkg, c) for c in mix]
    out = []
    with pkg.Server(max_active=16, **kw) as srv:
        report = srv.tuning
        ids = [submit_case(srv, c, u) for c, u in zip(mix, us)]
        for rid in ids:
            r = srv.wait(rid, timeout=600)
            assert r["status"] == 0, r
            out.append((srv.fields(rid), srv.stats_rows(rid)))
    return us, out, report


@pytest.mark.parametrize("kw", [dict(class_forms=1), dict(class_forms=2), dict(autotune=True)])
def test_class_forms_compute_the_same_step(gpu_pkg, kw):
    us, base, _ = _run_mix(gpu_pkg, FORM_MIX)
    _, got, report = _run_mix(gpu_pkg, FORM_MIX, **kw)
    if kw.get("autotune"):
        for n in (32, 48, 64, 96, 128):
            assert f"n={n} " in report, report
    for case, u, (fb, sb), (fg, sg) in zip(FORM_MIX, us, base, got):
        for c in range(3):
            assert np.linalg.norm(fg[c] - fb[c]) <= 1e-5 * np.linalg.norm(fb[c]), (case, c)
        assert sg.shape == sb.shape
        assert np.allclose(sg, sb, rtol=1e-5, atol=1e-6 * np.abs(sb).max()), case
    # against the FP64 oracle
    for case, u, (fg, _) in list(zip(FORM_MIX, us, got))[:3]:
        n, les, integ, adaptive, nt, seed = case
        ref = OracleSimulation(Params.from_global(gdict(n, les, integ, adaptive)), u)
        ref.initialize()
        ref.run(nt)
        ur = ref.u_physical()
        for c in range(3):
            assert np.linalg.norm(fg[c] - ur[c]) <= 1e-4 * np.linalg.norm(ur[c]), (case, c)
