"""Benchmark: steps/s of the pseudo-spectral solver step, forced isotropic DNS 256^3.

Workload: seeded random-phase, divergence-free field with E(k) ~ k^4 exp(-2 (k/k0)^2),
k0 = 4, u_rms = 1; isotropic band forcing |k| <= 2.5 at constant power eps = 0.1;
nu = 1e-3; AB3 with adaptive dt (CFL 0.5); 2/3 dealiasing; stats every 100 steps. A step
is one advance_in_time! (one CUDA-graph launch of the whole step).

The headline value is the FP64 plain form: the reference's own arithmetic, so it compares
like for like with the FP64 reference arm (--impl reference). The FP32 chosen form is
timed beside it (key "fp32") with its error against FP64 after 10 steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference] [--grid n]

N > 1 runs under torchrun as independent replicas (one per GPU, no collective on the data
path); value = steps of all ranks / max time over ranks.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "steps/s at 256\u00b3 FP32 vs FP64 GPU (stated L2 err); batched solves/s, p50/p99"
NU, K0, EPS, KF, CFL, DTSTAT = 1e-3, 4.0, 0.1, 2.5, 0.5, 100


def global_dict(n: int) -> dict:
    return {"nx": str(n), "ny": str(n), "nz": str(n), "xDomainSize": "1.0", "yDomainSize": "1.0",
            "zDomainSize": "1.0", "kinematicViscosity": str(NU), "dtStat": str(DTSTAT), "dtSpec": "1000000000",
            "writeTime": "1000000000", "velocityTimeStep": "Adams_Bashforth3rdO", "variableTimestepFlag": "true",
            "cfl": str(CFL), "dt": "0.001", "forcing": "isotropicBand", "forcingPower": str(EPS),
            "forcingKf": str(KF)}


def workload_name(n: int) -> str:
    return (f"forced isotropic DNS {n}^3: random-phase E(k)~k^4 exp(-2(k/4)^2) u_rms=1, band forcing "
            f"|k|<=2.5 eps=0.1, nu=1e-3, AB3 CFL 0.5, 2/3 dealias, stats every {DTSTAT} steps")


# ---------------------------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi sampling during the timed region (clocks and throttle reasons)."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------------- helpers
def measured_peaks() -> tuple[float, str]:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except (KeyError, ValueError):
            pass
    return 6800.0, "fallback"


def ncu_traffic(kernel: str, n: int, prec: str, name: str = "traffic.txt") -> float | None:
    """Per-launch DRAM bytes of a kernel from the committed ncu summary (profiles/traffic.txt),
    or another per-launch figure of the same format (profiles/fp64_instructions.txt)."""
    p = ROOT / "profiles" / name
    if not p.exists():
        return None
    for ln in p.read_text().splitlines():
        f = ln.split()
        if len(f) >= 4 and not ln.startswith("#") and f[0] == kernel and f[1] == str(n) and f[2] == prec:
            return float(f[3])
    return None


def model_bytes(n: int, elem: int) -> dict[str, float]:
    """Effective-bandwidth byte model of the velocity-only step, per pass.

    A = (n/2+1) n^2 complex elements of `elem` bytes (one full half-spectrum component).
    Each component 3D transform costs three sweeps of (read A + write A); the step runs 6
    inverse (u, w) and 3 forward (u x w) transforms; the integrator reads u, N, fm1, fm2
    and writes u for each of 3 components (5A each). Pointwise work is counted as fused.
    Per pass: z and y sweeps of the inverse transforms 12A each, x sweeps of all nine 18A,
    forward y and z sweeps 6A each, update 15A: 69A per step.
    """
    A = (n // 2 + 1) * n * n * elem
    return {"inv_z": 12 * A, "inv_y": 12 * A, "x_pass": 18 * A, "fwd_y": 6 * A, "fwd_z": 6 * A, "update": 15 * A,
            "step": 69 * A}


def retained(n: int) -> tuple[int, int]:
    """Retained kx count Mx and retained ky (= kz) count NYR of the 2/3 rule on n points."""
    mx = int(math.floor((2.0 / 3.0) * (n // 2) + 1e-12)) + 1
    return mx, 2 * mx - 1


def algorithmic_bytes(n: int, elem: int) -> dict[str, float]:
    """Minimal bytes each pass of the velocity-only step must move (retained modes only):
    what it has to read and write once, with nothing re-read.

    C = Mx*NYR*NZR (compact spectral component), V = Mx*NYR*n (after the z pass),
    U = Mx*n*n (after the y pass), complex elements of `elem` bytes. inv_z reads u (3C)
    and writes u, w (6V); inv_y 6V -> 6U; the x pass 6U -> 3U; fwd_y 3U -> 3V; fwd_z
    3V -> 3C; the update reads u, N, fm1, fm2 and writes u and the new rhs (18C).
    """
    mx, nr = retained(n)
    C, V, U = mx * nr * nr * elem, mx * nr * n * elem, mx * n * n * elem
    k = {"inv_z": 3 * C + 6 * V, "inv_y": 6 * V + 6 * U, "x_pass": 6 * U + 3 * U, "fwd_y": 3 * U + 3 * V,
         "fwd_z": 3 * V + 3 * C, "update": 18 * C}
    k["step"] = sum(k.values())
    return k


def algorithmic_flops(n: int) -> dict[str, float]:
    """Floating-point operations of the transforms each pass performs (velocity-only step),
    pruned to the retained modes like the kernels: 5 L log2 L per complex line of length L,
    2.5 L log2 L per real line. The x pass transforms 9 real fields on all n^2 (y,z) lines;
    the y and z passes only the Mx retained kx columns (and inv_z / fwd_z only the NYR
    retained ky rows). Pointwise products, projections and the update are not counted."""
    mx, nr = retained(n)
    lg = math.log2(n)
    cl = 5.0 * n * lg
    f = {"x_pass": 9 * n * n * 2.5 * n * lg, "inv_y": 6 * mx * n * cl, "inv_z": 6 * mx * nr * cl,
         "fwd_y": 3 * mx * n * cl, "fwd_z": 3 * mx * nr * cl}
    f["step"] = sum(f.values())
    return f


def dist_setup(args, backend: str = "nccl"):
    """Replicas: one process per GPU, no data-path collective. Only the timing uses the
    process group (a barrier around the timed region and a max over ranks)."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch
        import torch.distributed as dist
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    return world, rank, local, dist


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, v: float) -> float:
    if dist is None:
        return v
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_rate(dist, world: int, steps: int, ms_local: float) -> tuple[float, float]:
    """Whole-job steps/s of independent replicas: all ranks' steps over the slowest
    rank's time. Returns (steps/s, max ms)."""
    ms = max_over_ranks(dist, ms_local)
    return steps * world / (ms / 1e3), ms


def cuda_sync():
    try:
        import torch
        if torch.cuda.is_available():
            torch.cuda.synchronize()
    except ImportError:
        pass


# ---------------------------------------------------------------------------------- arms
def cpu_reference_rate(n: int, budget_s: float, max_steps: int, warmup: int) -> tuple[float, int, int]:
    """The FP64 CPU oracle (a port of the reference step) on this host's cores."""
    import numpy as np
    import __graft_entry__ as ge
    from oracle.ffs_oracle import OracleSimulation, Params
    pkg = ge.load_package()
    u = pkg.random_spectrum(n, k0=K0, seed=2001)
    s = OracleSimulation(Params.from_global(global_dict(n)), u)
    s.initialize()
    for _ in range(warmup):
        s.advance()
    t0 = time.perf_counter()
    k = 0
    while k < max_steps:
        s.advance()
        k += 1
        if time.perf_counter() - t0 > budget_s:
            break
    dt = time.perf_counter() - t0
    cores = int(os.environ.get("FFS_ORACLE_WORKERS", os.cpu_count() or 1))
    del np
    return k / dt, k, cores


# ---------------------------------------------------------------------------------- serving
SERVE_SIZES = (32, 48, 64, 96, 128)
SERVE_RATE = 200.0   # mean Poisson arrivals per second
SERVE_BATCH_LAUNCHES = 6 * 11   # kernels per batched step: 6 size-class chains of 11 (one CUDA graph)


def serving_requests(R: int) -> list[dict]:
    """Seeded served-ensemble trace: Poisson arrivals (mean 200/s), n ~ U{32,48,64,96,128},
    k0 ~ U{2..6}, nu ~ logU[1e-3, 1e-2], nt ~ U{100..1000} AB3 steps (adaptive dt at the
    reference's default CFL 0.18), 50% Smagorinsky LES."""
    import numpy as np
    rng = np.random.default_rng(5000)
    t = np.cumsum(rng.exponential(1.0 / SERVE_RATE, size=R))
    out = []
    for i in range(R):
        n = int(rng.choice(SERVE_SIZES))
        k0 = int(rng.integers(2, 7))
        nu = float(10 ** rng.uniform(-3, -2))
        nt = int(rng.integers(100, 1001))
        les = bool(rng.random() < 0.5)
        out.append({"i": i, "t": float(t[i]), "n": n, "k0": k0, "nu": nu, "nt": nt, "les": les, "seed": 5000 + i})
    return out


def serve_global(r: dict) -> dict:
    n = str(r["n"])
    d = {"nx": n, "ny": n, "nz": n, "xDomainSize": "1.0", "yDomainSize": "1.0", "zDomainSize": "1.0",
         "kinematicViscosity": repr(r["nu"]), "dtStat": "50", "dtSpec": "1000000000", "writeTime": "1000000000",
         "velocityTimeStep": "Adams_Bashforth3rdO", "variableTimestepFlag": "true", "cfl": "0.18", "dt": "0.001"}
    if r["les"]:
        d.update({"lesModel": "Smagorinsky", "smagorinskyConstant": "0.17"})
    return d


def _pct(v, q):
    import numpy as np
    return float(np.percentile(np.asarray(v), q)) if len(v) else None


def queue_replay(reqs, service):
    """Completion times of requests served one at a time in arrival order."""
    end, lat = 0.0, []
    for r, s in zip(reqs, service):
        start = max(r["t"], end)
        end = start + s
        lat.append(end - r["t"])
    span = end - reqs[0]["t"] if service else 0.0
    return lat, span


def run_serving(pkg, R: int, seq_budget: float, device: int) -> dict:
    reqs = serving_requests(R)
    fields = [pkg.random_spectrum(r["n"], k0=float(r["k0"]), seed=r["seed"]) for r in reqs]
    total_steps = sum(r["nt"] for r in reqs)
    points = sum(r["nt"] * r["n"] ** 3 for r in reqs)
    with pkg.Server(device=device, memory_budget=120 << 30, max_active=256, autotune=True) as srv:
        tuning = srv.tuning   # the size classes' kernel forms, timed at create
        # warm-up: one short run per grid and model (module load, first allocations)
        warm = [srv.submit(serve_global(dict(r, nt=3)), fields[r["i"]], 3)
                for r in {(x["n"], x["les"]): x for x in reqs}.values()]
        for w in warm:
            srv.wait(w, 600)
            srv.release(w)
        before = srv.info()
        t0 = time.perf_counter()
        ids = []
        for r in reqs:
            delay = t0 + r["t"] - time.perf_counter()
            if delay > 0:
                time.sleep(delay)
            ids.append(srv.submit(serve_global(r), fields[r["i"]], r["nt"]))
        res, errors = [], []
        for i in ids:
            try:
                res.append(srv.wait(i, 3600))
            except pkg.FFSError as e:
                errors.append(str(e))
        info = srv.info()
    if not res:
        return {"error": errors[:3]}
    lat = [x["done_s"] - x["submit_s"] for x in res]
    span = max(x["done_s"] for x in res) - min(x["submit_s"] for x in res)
    batch_steps = info["batch_steps"] - before["batch_steps"]
    batched = {"solves_per_s": len(res) / span, "p50_s": _pct(lat, 50), "p99_s": _pct(lat, 99),
               "sim_steps_per_s": total_steps / span, "grid_point_updates_per_s": points / span,
               "wall_s": span, "batch_steps": batch_steps, "peak_active": info["peak_active"],
               "peak_bytes": info["peak_bytes"], "gpu_launches": batch_steps * SERVE_BATCH_LAUNCHES,
               "failed": len(errors), "errors": errors[:3], "tuning": tuning}
    out = {"workload": f"served ensemble: {R} requests, Poisson arrivals mean {SERVE_RATE:.0f}/s, n ~ U{{32..128}}, "
                       "k0 ~ U{2..6}, nu ~ logU[1e-3,1e-2], nt ~ U{100..1000} AB3 (CFL 0.18), 50% Smagorinsky, "
                       "FP32, 120 GB budget",
           "requests": R, "sim_steps": total_steps, "batched": batched}
    for prec in ("FP32", "FP64"):
        service, failed = [], 0
        t_all = time.perf_counter()
        for r in reqs:
            t = time.perf_counter()
            sim = pkg.Simulation(pkg.parameters(serve_global(r), precision=prec, device=device))
            try:
                sim.set_fields(*fields[r["i"]])
                sim.initialize()
                sim.advance_in_time(r["nt"])
            except pkg.FFSError:
                failed += 1     # e.g. a diverged run: it still occupied the GPU until it stopped
            sim.close()
            service.append(time.perf_counter() - t)
            if time.perf_counter() - t_all > seq_budget:
                break
        k = len(service)
        lat_s, span_s = queue_replay(reqs[:k], service)
        out[f"sequential_{prec.lower()}"] = {
            "requests_run": k, "failed": failed, "solves_per_s": (k - failed) / span_s if span_s > 0 else None,
            "p50_s": _pct(lat_s, 50),
            "p99_s": _pct(lat_s, 99), "mean_service_s": sum(service) / k if k else None,
            "note": "same requests one at a time through Simulation (plain single-simulation path), "
                    "arrival-order queue replayed with the measured service times"
                    + ("" if k == R else f"; first {k} requests within a {seq_budget:.0f} s budget")}
    return out


# ---------------------------------------------------------------------------------- other configurations
def workload_config(wl: str):
    """(global dict, n, precision of the timed arm, IC kind, description) of a configuration."""
    if wl == "tg64":
        d = {"nx": "64", "ny": "64", "nz": "64", "xDomainSize": "1.0", "yDomainSize": "1.0", "zDomainSize": "1.0",
             "kinematicViscosity": "0.0333333", "dtStat": "20", "dtSpec": "1000000000", "writeTime": "1000000000",
             "velocityTimeStep": "ETD3rdO", "variableTimestepFlag": "false", "dt": "0.05"}
        # AB3 treats viscosity explicitly: nu k_max^2 dt = 0.0333 * 3 * 21^2 * 0.05 = 2.2 is far outside
        # its stability interval (-6/11, 0), so AB3 at this dt diverges in a few steps. ETD3 (the
        # reference's default integrator) integrates the viscous term exactly.
        return d, 64, "FP64", "tg", ("Taylor-Green vortex 64^3 FP64 (u1 = cos x sin y sin z, u2 = -sin x cos y "
                                     "sin z, u3 = 0), nu = 0.0333333, dt = 0.05, ETD3 (AB3 is viscously "
                                     "unstable at this dt), stats every 20 steps")
    if wl == "les128":
        d = {"nx": "128", "ny": "128", "nz": "128", "xDomainSize": "1.0", "yDomainSize": "1.0", "zDomainSize": "1.0",
             "kinematicViscosity": "5e-4", "dtStat": "50", "dtSpec": "50", "writeTime": "1000000000",
             "velocityTimeStep": "ETD3rdO", "variableTimestepFlag": "true", "cfl": "0.18", "dt": "0.001",
             "lesModel": "Smagorinsky", "smagorinskyConstant": "0.17", "filterWidth": repr(2 * math.pi / 128),
             "densityStratification": "true", "zAcceleration": "1", "referenceDensity": "1",
             "densityGradient": "1", "Pr": "1"}
        return d, 128, "FP32", "random3", ("stably stratified Boussinesq LES 128^3 FP32: random-phase k0 = 3, "
                                           "rho' = 0, N = 1, Pr = 1, Smagorinsky Cs = 0.17, Delta = 2 pi/128, "
                                           "nu = 5e-4, ETD3 (CFL 0.18), stats and spectra every 50 steps")
    if wl == "dns1024":
        d = {"nx": "1024", "ny": "1024", "nz": "1024", "xDomainSize": "1.0", "yDomainSize": "1.0",
             "zDomainSize": "1.0", "kinematicViscosity": "2e-4", "dtStat": "100", "dtSpec": "1000000000",
             "writeTime": "1000000000", "velocityTimeStep": "Adams_Bashforth3rdO", "variableTimestepFlag": "true",
             "cfl": "0.5", "dt": "0.0001", "forcing": "isotropicBand", "forcingPower": "0.1", "forcingKf": "2.5",
             "hyperViscosity": "true", "hyperViscosityCoefficient": "1e-12", "hyperViscosityM": "2"}
        return d, 1024, "FP32", "modes8", ("large single-instance DNS 1024^3 FP32: random-phase k0 = 8 (spectral "
                                           "generator, modes |k_i| <= 48), band forcing eps = 0.1, nu = 2e-4, "
                                           "hyperviscosity 1e-12 k^4, AB3 CFL 0.5")
    raise ValueError(wl)


def make_sim(pkg, d, prec, ic, n, device, autotune=1):
    p = pkg.parameters(d, precision=prec, device=device)
    p.autotune = autotune
    sim = pkg.Simulation(p)
    if ic == "tg":
        sim.set_fields(*pkg.taylor_green(n))
    elif ic == "random3":
        sim.set_fields(*pkg.random_spectrum(n, k0=3.0, seed=3001))
    else:
        from importlib import import_module
        f = import_module(pkg.__name__ + ".fields")
        kc = 48
        box = f.random_spectrum_modes(n, 8.0, 4001, kc)
        for c in range(3):
            sim.set_spectral(c, f.embed_half_spectrum(box[c], n, kc))
    sim.initialize()
    return sim


def run_large(pkg, device: int, steps: int, autotune: int) -> dict:
    """The large single-instance configuration (DNS 1024^3 + hyperviscosity, FP32) measured
    inside the default run: K graph replays after 3 warm-up steps, per-kernel event times
    and their HBM fractions against the 69A effective-bytes model, DRAM traffic per launch
    from the committed ncu captures (profiles/traffic.txt; 1024^3 rows scaled from the
    512^3 capture, see the file), clocks sampled during the timed replays."""
    d, n, prec, ic, desc = workload_config("dns1024")
    try:
        sim = make_sim(pkg, d, prec, ic, n, device, autotune)
    except pkg.FFSError as e:
        return {"workload": desc, "error": str(e)}
    sim.advance_in_time(3)
    with ClockSampler(device) as clk:
        ms = sim.time_steps(steps)
    nprof = 3
    prof = sim.profile_kernels(nprof)
    out = {"workload": desc, "value": steps / (ms / 1e3), "unit": "steps/s", "steps": steps, "warmup": 3,
           "ms_per_step": ms / steps, "grid_point_updates_per_s": steps / (ms / 1e3) * n ** 3,
           "device_gb": sim.device_bytes / 1e9, "kernels_ms_per_step": {k: v / nprof for k, v in prof.items()},
           "gpu_launches": sim.launches_per_step * (steps + nprof), "clocks": clk.summary(), "tuning": sim.tuning}
    sim.close()
    peak, kind = measured_peaks()
    sb = model_bytes(n, 8)
    roof = {"bound": "hbm", "unit": "GB/s", "peak": peak, "peak_source": kind,
            "bytes_model": "69A per step, A = (n/2+1) n^2 complex FP32 (hyperviscosity adds no passes)",
            "step_frac": sb["step"] / (ms / steps / 1e3) / 1e9 / peak, "per_kernel": {}}
    for k in ("inv_z", "inv_y", "x_pass", "fwd_y", "fwd_z", "update"):
        if prof.get(k, 0) <= 0:
            continue
        t = prof[k] / nprof / 1e3
        e = {"ms": t * 1e3, "model_frac": sb[k] / t / 1e9 / peak}
        tr = ncu_traffic(k, n, "fp32")
        if tr:
            e["traffic"] = tr
            e["dram_frac"] = tr / t / 1e9 / peak
        roof["per_kernel"][k] = e
    out["roofline"] = roof
    return out


def run_workload(args):
    """One JSON line for a configuration other than the headline 256^3 run."""
    import numpy as np
    import __graft_entry__ as ge
    pkg = ge.load_package()
    pkg.load()
    d, n, prec, ic, desc = workload_config(args.workload)
    world, rank, local, dist = dist_setup(args)
    sim = make_sim(pkg, d, prec, ic, n, local, 0 if args.no_autotune else 1)
    tuning = sim.tuning
    sim.advance_in_time(max(args.warmup, 3))
    with ClockSampler(local) as clk:
        ms = sim.time_steps(args.steps)
    rate = args.steps / (ms / 1e3)
    nprof = max(3, min(10, args.steps))
    prof = sim.profile_kernels(nprof)
    dev_bytes = sim.device_bytes
    launches = sim.launches_per_step * args.steps
    sim.close()
    out = {"metric": METRIC, "value": rate, "unit": "steps/s", "n_gpus": 1, "steps": args.steps,
           "warmup": max(args.warmup, 3), "ms_per_step": ms / args.steps, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32" if prec == "FP32" else "f64", "data": "synthetic",
           "config": {"workload": desc, "grid": n, "l2": f"{dev_bytes / 1e9:.2f} GB resident per GPU"},
           "grid_point_updates_per_s": rate * n ** 3,
           "kernels_ms_per_step": {k: v / nprof for k, v in prof.items()}, "clocks": clk.summary(),
           "gpu_launches": launches, "tuning": tuning}
    peak, kind = measured_peaks()
    elem = 8 if prec == "FP32" else 16
    A = (n // 2 + 1) * n * n * elem
    ntr = 23 if "lesModel" in d else 9        # component transforms per step
    nint = 4 if "densityStratification" in d else 3
    b_alg = (6 * ntr + 5 * nint) * A
    out["roofline"] = {"bound": "hbm", "step_algorithmic_bytes": b_alg, "bytes_model":
                       f"{6 * ntr + 5 * nint}A per step ({ntr} component transforms x 6A + {nint} integrated "
                       f"fields x 5A), A = (n/2+1) n^2 complex", "achieved": b_alg / (ms / args.steps / 1e3) / 1e9,
                       "peak": peak, "unit": "GB/s", "peak_source": kind}
    out["roofline"]["frac"] = out["roofline"]["achieved"] / peak
    if ntr == 9:   # velocity-only: the per-pass split of the 69A model
        sb = model_bytes(n, elem)
        out["roofline"]["per_kernel_frac"] = {k: sb[k] / (prof[k] / nprof / 1e3) / 1e9 / peak
                                              for k in sb if k in prof and prof[k] > 0}
    if prec == "FP32":
        # FP64 plain form on the same initial state, and the FP32 error after 10 steps
        try:
            a, b = make_sim(pkg, d, "FP32", ic, n, local), make_sim(pkg, d, "FP64", ic, n, local)
            a.advance_in_time(10)
            b.advance_in_time(10)
            err = 0.0
            for c in range(3):
                bb = b.spectral(c)
                err = max(err, float(np.linalg.norm(a.spectral(c) - bb) / np.linalg.norm(bb)))
                del bb
            a.close()
            k64 = 3 if n >= 1024 else 10
            ms64 = b.time_steps(k64)
            b.close()
            out["fp64"] = {"value": k64 / (ms64 / 1e3), "unit": "steps/s", "steps": k64}
            out["fp32_vs_fp64_rel_l2_10_steps"] = err
        except pkg.FFSError as e:
            out["fp64"] = {"error": str(e)}
    if n <= 128 and not args.no_cpu:
        from oracle.ffs_oracle import OracleSimulation, Params
        u = pkg.taylor_green(n) if ic == "tg" else pkg.random_spectrum(n, k0=3.0, seed=3001)
        o = OracleSimulation(Params.from_global(d), u)
        o.initialize()
        o.advance()
        t0 = time.perf_counter()
        k = 0
        while time.perf_counter() - t0 < args.cpu_budget and k < 200:
            o.advance()
            k += 1
        v = k / (time.perf_counter() - t0)
        out["cpu_baseline"] = {"value": v, "unit": "steps/s", "cores": os.cpu_count(), "kind": "port",
                               "sample": f"{k} steps of the same workload, FP64 numpy/pocketfft oracle"}
    print(json.dumps(out), flush=True)
    return 0


def run_reference_arm(args):
    world, rank, local, dist = dist_setup(args)
    if rank != 0:
        return 0
    n = args.grid
    rate, k, cores = cpu_reference_rate(n, budget_s=args.ref_budget, max_steps=args.steps,
                                        warmup=min(args.warmup, 1))
    line = {"impl": "reference", "metric": METRIC, "value": rate, "unit": "steps/s", "n_gpus": args.gpus,
            "steps": k, "warmup": min(args.warmup, 1), "ms_per_step": 1e3 / rate, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": workload_name(n), "grid": n, "implementation": "FP64 CPU port of the reference "
                       "step (numpy + scipy.fft pocketfft); the Julia/FFTW reference cannot run on this box"},
            "cpu_baseline": {"value": rate, "unit": "steps/s", "cores": cores, "kind": "port",
                             "sample": f"{k} timed steps of the {n}^3 workload after 1 warm-up step "
                                       f"(budget {args.ref_budget:.0f} s)"},
            "e2e": {"value": rate, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def kernel_roofline_hbm(prof: dict, nprof: int, n: int, elem: int, prec: str, peak: float, peak_kind: str,
                        ms_step: float) -> dict:
    """HBM roofline of the dominant kernel of a form: achieved = the kernel's retained-mode
    algorithmic bytes (what it must read and write once) / its event-timed duration;
    traffic = its ncu DRAM bytes per launch (profiles/traffic.txt); dram_frac = traffic /
    duration / peak. The 69A effective-bandwidth figure is kept as a labelled extra."""
    alg = algorithmic_bytes(n, elem)
    sb = model_bytes(n, elem)
    cand = {k: v for k, v in prof.items() if k in alg}
    top = max(cand, key=cand.get)
    top_ms = prof[top] / nprof
    achieved = alg[top] / (top_ms / 1e3) / 1e9
    traffic = ncu_traffic(top, n, prec)
    r = {"bound": "hbm", "kernel": top, "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
         "traffic": traffic, "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
         "algorithmic_bytes_per_launch": alg[top],
         "bytes_model": "retained-mode minimum per pass (C = Mx NYR NZR, V = Mx NYR n, U = Mx n^2 complex)",
         "step_algorithmic_bytes": alg["step"], "step_frac": alg["step"] / (ms_step / 1e3) / 1e9 / peak,
         "per_kernel_frac": {k: alg[k] / (prof[k] / nprof / 1e3) / 1e9 / peak for k in alg
                             if k != "step" and prof.get(k, 0) > 0},
         "effective_69A_frac": sb.get(top, 0.0) / (top_ms / 1e3) / 1e9 / peak}
    if traffic:
        r["dram_achieved"] = traffic / (top_ms / 1e3) / 1e9
        r["dram_frac"] = r["dram_achieved"] / peak
    return r


def run_engine_arm(args):
    import numpy as np
    import __graft_entry__ as ge
    world, rank, local, dist = dist_setup(args)
    pkg = ge.load_package()
    L = pkg.load()
    n = args.grid
    d = global_dict(n)
    u = pkg.random_spectrum(n, k0=K0, seed=2001)

    def make(prec, autotune=None):
        p = pkg.parameters(d, precision=prec, device=local)
        p.autotune = (0 if args.no_autotune else 1) if autotune is None else autotune
        sim = pkg.Simulation(p)
        sim.set_fields(*u)
        sim.initialize()
        return sim

    # --- headline: the FP64 plain form (the reference's arithmetic), inputs resident in HBM
    sim64 = make("FP64")
    tuning64 = sim64.tuning
    sim64.advance_in_time(max(args.warmup, 3))
    cuda_sync()
    barrier(dist)
    with ClockSampler(local) as clk:
        ms = sim64.time_steps(args.steps)
    cuda_sync()
    barrier(dist)
    steps_s, ms = replica_rate(dist, world, args.steps, ms)
    launches = sim64.launches_per_step * args.steps
    nprof = max(3, min(10, args.steps))
    prof64 = sim64.profile_kernels(nprof)
    dev_bytes = sim64.device_bytes
    sim64.close()

    # --- the FP32 chosen form on the same initial fields
    sim = make("FP32")
    tuning32 = sim.tuning
    sim.advance_in_time(max(args.warmup, 3))
    k32 = max(20, min(args.steps * 10, 1000))
    ms32 = sim.time_steps(k32)
    nprof32 = max(5, min(20, args.steps))
    prof32 = sim.profile_kernels(nprof32)
    launches += sim.launches_per_step * k32
    sim.close()

    # --- FP32 vs FP64 error after 10 steps (same initial fields; the FP64 engine matches
    # the oracle to 1e-12 at this size, tests/test_gpu_configs.py)
    a, b = make("FP32", 0), make("FP64", 0)
    a.advance_in_time(10)
    b.advance_in_time(10)
    err = max(float(np.linalg.norm(a.spectral(c) - b.spectral(c)) / np.linalg.norm(b.spectral(c)))
              for c in range(3))
    a.close()
    b.close()

    # --- end to end through the public API with host buffers (the engine already created:
    # allocation and plans are one-time setup): set_fields from host memory, initialize!,
    # K steps, the run's tail, the Stats rows and the final fields back to the host
    def e2e(prec):
        host = [np.ascontiguousarray(x) for x in u]
        p = pkg.parameters(d, precision=prec, device=local)
        e = pkg.Simulation(p)
        cuda_sync()
        t0 = time.perf_counter()
        e.set_fields(*host)
        e.initialize()
        e.advance_in_time(args.steps)
        e.finalize()
        rows = e.stats_rows()
        out = e.fields()
        t1 = time.perf_counter()
        e.close()
        return max_over_ranks(dist, t1 - t0), rows.nbytes + sum(x.nbytes for x in out), sum(x.nbytes for x in host)

    e2e_s, d2h, h2d = e2e("FP64")
    e2e_rate = args.steps * world / e2e_s
    e2e32_s, _, _ = e2e("FP32")
    launches += (sim.launches_per_step + 1) * (args.steps + 2)

    # --- the FP64 arithmetic peak of this GPU (roofline denominator of the FP64 form)
    fma_tf, add_tf = ctypes.c_double(), ctypes.c_double()
    rc = L.ffs_measure_fp64_peak(local, ctypes.byref(fma_tf), ctypes.byref(add_tf))
    fp64_peak = fma_tf.value if rc == 0 else None

    if rank != 0:
        return 0
    peak, peak_kind = measured_peaks()
    ms_step = ms / args.steps
    fl = algorithmic_flops(n)
    cand = {k: v for k, v in prof64.items() if k in fl}
    top64 = max(cand, key=cand.get)
    top64_ms = prof64[top64] / nprof
    tr64 = ncu_traffic(top64, n, "fp64")
    roof64 = {"bound": "fp64", "kernel": top64, "achieved": fl[top64] / (top64_ms / 1e3) / 1e12,
              "peak": fp64_peak, "unit": "TFLOP/s",
              "frac": (fl[top64] / (top64_ms / 1e3) / 1e12 / fp64_peak) if fp64_peak else None,
              "traffic": tr64,
              "peak_source": "measured in this run: ffs_measure_fp64_peak (FP64 FMA chains on every SM, 2 flops "
                             "per FMA); no FP64 figure is in MEASURED_PEAKS.json",
              "fp64_add_peak": add_tf.value if rc == 0 else None,
              "flop_model": "pruned transform flops per pass: 5 L log2 L per complex line, 2.5 L log2 L per real "
                            "line, retained columns only",
              "algorithmic_flops_per_launch": fl[top64],
              "step_algorithmic_flops": fl["step"],
              "step_frac": (fl["step"] / (ms_step / 1e3) / 1e12 / fp64_peak) if fp64_peak else None,
              "per_kernel_frac": ({k: fl[k] / (prof64[k] / nprof / 1e3) / 1e12 / fp64_peak for k in fl
                                   if k != "step" and prof64.get(k, 0) > 0} if fp64_peak else None),
              "hbm": kernel_roofline_hbm(prof64, nprof, n, 16, "fp64", peak, peak_kind, ms_step)}
    if tr64:
        roof64["dram_frac"] = tr64 / (top64_ms / 1e3) / 1e9 / peak
    ins64 = ncu_traffic(top64, n, "fp64", "fp64_instructions.txt")
    if ins64 and fp64_peak:
        # FP64-pipe occupancy: the kernel's counted FP64 warp instructions (one ncu capture)
        # per event-timed launch against the pipe's rate at the measured peak (1 FMA = 2 flops)
        roof64["fp64_pipe_frac"] = ins64 * 32 / (top64_ms / 1e3) / (fp64_peak * 1e12 / 2)
        roof64["fp64_warp_instructions_per_launch"] = ins64
        if rc == 0 and add_tf.value > 0:
            # against the add (and multiply) instruction rate, the form of most butterfly work
            roof64["fp64_pipe_frac_add_rate"] = ins64 * 32 / (top64_ms / 1e3) / (add_tf.value * 1e12)
    ms32_step = ms32 / k32
    roof32 = kernel_roofline_hbm(prof32, nprof32, n, 8, "fp32", peak, peak_kind, ms32_step)
    cpu_rate, cpu_k, cores = (None, 0, 0)
    if not args.no_cpu:
        cpu_rate, cpu_k, cores = cpu_reference_rate(n, budget_s=args.cpu_budget, max_steps=50, warmup=1)
    clocks = clk.summary()
    line = {
        "metric": METRIC, "value": steps_s, "unit": "steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": ms_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": workload_name(n), "grid": n,
                   "precision": "FP64 plain form (the reference's arithmetic); the FP32 chosen form is in fp32",
                   "parallelism": f"replicas x{world}",
                   "l2": f"inputs larger than L2: {dev_bytes / 1e9:.2f} GB resident per GPU (FP64)"},
        "grid_point_updates_per_s": steps_s * n ** 3,
        "kernels_ms_per_step": {k: v / nprof for k, v in prof64.items()},
        "roofline": roof64,
        "fp32": {"value": k32 / (ms32 / 1e3) * world, "unit": "steps/s", "ms_per_step": ms32_step, "steps": k32,
                 "speedup_vs_fp64": (k32 / (ms32 / 1e3)) / (steps_s / world),
                 "rel_l2_vs_fp64_10_steps": err,
                 "precision": "FP32 transforms/products/updates; FP64 twiddles, phi-coefficients and reductions",
                 "kernels_ms_per_step": {k: v / nprof32 for k, v in prof32.items()},
                 "roofline": roof32,
                 "e2e": {"value": args.steps * world / e2e32_s, "unit": "steps/s"},
                 "tuning": tuning32},
        "cpu_baseline": ({"value": cpu_rate, "unit": "steps/s", "cores": cores, "kind": "port",
                          "sample": f"{cpu_k} steps of the same {n}^3 workload, FP64 numpy/pocketfft oracle"}
                         if cpu_rate else None),
        "e2e": {"value": e2e_rate, "unit": "steps/s", "h2d_bytes_per_step": h2d / args.steps,
                "d2h_bytes_per_step": d2h / args.steps,
                "includes": "set_fields from host memory, initialize!, advance_in_time(K), run tail, stats rows "
                            "and final fields to host memory (FP64; engine creation is one-time setup, outside)"},
        "clocks": clocks,
        "gpu_launches": launches,
        "tuning": tuning64,
    }
    if args.serve_requests > 0:
        line["serving"] = run_serving(pkg, args.serve_requests, args.serve_seq_budget, local)
        line["gpu_launches"] += line["serving"].get("batched", {}).get("gpu_launches", 0)
    if args.large_steps > 0 and world == 1:
        line["dns1024"] = run_large(pkg, local, args.large_steps, 0 if args.no_autotune else 1)
        line["gpu_launches"] += line["dns1024"].get("gpu_launches", 0)
    print(json.dumps(line), flush=True)
    return 0


def fp32_error_run(pkg, name: str, nt: int, device: int) -> dict:
    """FP32 chosen form against the FP64 plain form over a configuration's full run, from
    the same initial state: relative differences of the energy (k), dissipation (diss) and
    total dissipation (tdiss) series of the Stats rows (every dtStat steps, plus the run's
    tail) and of the final u spectrum; the per-component relative L2 after 10 steps."""
    import numpy as np
    if name == "dns256":
        d, n, ic = dict(global_dict(256), dtStat="100"), 256, "dns256"
    else:
        d, n, _, ic, _ = workload_config(name)
    d = dict(d, dtSpec="1000000000")
    out = {"steps": nt, "grid": n, "dt_stat": int(d["dtStat"])}

    def make(prec):
        if ic == "dns256":
            p = pkg.parameters(d, precision=prec, device=device)
            sim = pkg.Simulation(p)
            sim.set_fields(*pkg.random_spectrum(n, k0=K0, seed=2001))
            sim.initialize()
            return sim
        return make_sim(pkg, d, prec, ic, n, device, autotune=0)

    runs = {}
    for prec in ("FP32", "FP64"):
        sim = make(prec)
        sim.advance_in_time(10)
        u10 = [sim.spectral(c) for c in range(3)]
        t0 = time.perf_counter()
        sim.advance_in_time(nt - 10)
        sim.finalize()
        wall = time.perf_counter() - t0
        rows = sim.stats_rows()
        H, V = sim.spectrum()
        runs[prec] = (u10, rows, H, V, wall, sim.header.split(","))
        sim.close()
    (a10, ra, Ha, Va, wa, names), (b10, rb, Hb, Vb, wb, _) = runs["FP32"], runs["FP64"]
    out["rel_l2_10_steps"] = [float(np.linalg.norm(a10[c] - b10[c]) / np.linalg.norm(b10[c])) for c in range(3)]
    out["rows"] = int(rb.shape[0])
    out["final_iteration"] = int(rb[-1, 0])
    cols = ["k", "diss", "tdiss"] + (["rhop2"] if "rhop2" in names else [])
    for c in cols:
        j = names.index(c)
        ok = np.abs(rb[:, j]) > 1e-12 * np.abs(rb[:, j]).max()   # rows where the quantity is not ~0 (rho = 0 at t = 0)
        rd = np.abs(ra[ok, j] - rb[ok, j]) / np.abs(rb[ok, j])
        out[f"{c}_max_rel_diff"] = float(rd.max())
        out[f"{c}_final_rel_diff"] = float(rd[-1])
    # the spectrum's bins that hold energy (above 1e-12 of its peak)
    sl = np.abs(Hb) > 1e-12 * np.abs(Hb).max()
    sl[0] = False
    out["specH_final_max_rel_diff_energetic_bins"] = float((np.abs(Ha[sl] - Hb[sl]) / np.abs(Hb[sl])).max())
    out["specH_final_energetic_bins"] = int(sl.sum())
    out["specH_final_rel_l2"] = float(np.linalg.norm(Ha - Hb) / np.linalg.norm(Hb))
    out["specV_final_rel_l2"] = float(np.linalg.norm(Va - Vb) / np.linalg.norm(Vb))
    out["wall_s"] = {"FP32": wa, "FP64": wb}
    return out


def run_fp32_error(args):
    """--fp32-error: the FP32 chosen form's stated error over every configuration's full run."""
    import __graft_entry__ as ge
    pkg = ge.load_package()
    pkg.load()
    plan = {"dns256": 2000, "les128": 5000, "dns1024": 200}
    want = args.configs.split(",") if args.configs else list(plan)
    res = {}
    for name in want:
        try:
            res[name] = fp32_error_run(pkg, name, plan[name], 0)
        except pkg.FFSError as e:
            res[name] = {"error": str(e)}
        print(json.dumps({name: res[name]}), flush=True)
    print(json.dumps({"fp32_error": res}), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--grid", type=int, default=256)
    ap.add_argument("--workload", default="dns256", choices=["dns256", "tg64", "les128", "dns1024"],
                    help="dns256: the headline run; the others print one line for that configuration")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--fp32-error", action="store_true",
                    help="FP32 vs FP64 over each configuration's full run (not part of the default bench)")
    ap.add_argument("--configs", default="", help="with --fp32-error: comma-separated subset of dns256,les128,dns1024")
    ap.add_argument("--no-autotune", action="store_true", help="default launch shapes instead of the tuned ones")
    ap.add_argument("--cpu-budget", type=float, default=20.0)
    ap.add_argument("--ref-budget", type=float, default=120.0)
    ap.add_argument("--serve-requests", type=int, default=64, help="served-ensemble requests (0: skip)")
    ap.add_argument("--serve-seq-budget", type=float, default=60.0,
                    help="seconds for each one-at-a-time baseline of the served ensemble")
    ap.add_argument("--large-steps", type=int, default=10,
                    help="timed steps of the 1024^3 FP32 configuration in the default run (0: skip)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference_arm(args)
    if args.fp32_error:
        return run_fp32_error(args)
    if args.workload != "dns256":
        return run_workload(args)
    return run_engine_arm(args)


if __name__ == "__main__":
    sys.exit(main())
