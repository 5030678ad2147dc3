"""Host-side mirror of the reference's simulation API over libffs.

``Simulation`` owns one engine handle (one GPU simulation). ``run_simulation`` mirrors
``run_simulation()`` (src/FluidFlowSimulation.jl:23-65): it reads ``global`` and the
``u1.$start``/``u2``/``u3`` (+``rho``) files, runs ``initialize!`` and the time loop on
the GPU, and writes Stats.txt, the u spectra and the field files in the reference
formats.
"""
from __future__ import annotations

import ctypes
from ctypes import byref, c_double, c_int32, c_int64, c_void_p
from pathlib import Path

import numpy as np

from . import fields as _fields
from . import scales as _scales
from ._lib import FFS_FP32, FFSError, FFSParams, load
from .globalfile import parameters, readglobal

_D = ctypes.POINTER(c_double)


def _ptr(a: np.ndarray | None):
    if a is None:
        return None
    return a.ctypes.data_as(_D)


def julia_float(x: float) -> str:
    """Print a Float64 the way Julia's ``print`` does (shortest round-trip digits)."""
    if x != x:
        return "NaN"
    if x in (float("inf"), float("-inf")):
        return "Inf" if x > 0 else "-Inf"
    r = repr(float(x))
    if "e" in r:
        m, e = r.split("e")
        if "." not in m:
            m += ".0"
        return f"{m}e{int(e)}"
    if "." not in r:
        r += ".0"
    return r


class Simulation:
    """One GPU simulation (the reference's ``Simulation`` object, src/simulationtypes.jl:45-100)."""

    def __init__(self, params: FFSParams):
        self._L = load()
        self.params = params
        h = c_void_p()
        rc = self._L.ffs_create(byref(params), byref(h))
        if rc != 0:
            raise FFSError(rc, self._L.ffs_last_error(None).decode())
        self._h = h
        self.nx, self.ny, self.nz = params.nx, params.ny, params.nz
        self.ncols = self._L.ffs_stats_ncols(h)
        self.rec_ncols = self._L.ffs_record_ncols(h)
        buf = ctypes.create_string_buffer(4096)
        self._check(self._L.ffs_stats_header(h, buf, 4096))
        self.header = buf.value.decode()
        lh, lv = c_int32(), c_int32()
        self._check(self._L.ffs_spectrum_lengths(h, byref(lh), byref(lv)))
        self.lenH, self.lenV = lh.value, lv.value
        self.has_density = bool(params.density or params.passive_scalar)   # a fourth field
        self.scalar_name = "scalar" if params.passive_scalar else "rho"

    @classmethod
    def from_global(cls, d: dict, precision: str | None = None, device: int = 0) -> "Simulation":
        return cls(parameters(d, precision=precision, device=device))

    # ---------------------------------------------------------------- plumbing
    def _check(self, rc: int):
        if rc != 0:
            raise FFSError(rc, self._L.ffs_last_error(self._h).decode())

    def close(self):
        if getattr(self, "_h", None):
            self._L.ffs_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ---------------------------------------------------------------- reference API
    def set_fields(self, u1, u2, u3, rho=None, layout: int = 0):
        a = [np.ascontiguousarray(x, dtype=np.float64) for x in (u1, u2, u3)]
        r = None if rho is None else np.ascontiguousarray(rho, dtype=np.float64)
        self._check(self._L.ffs_set_fields(self._h, _ptr(a[0]), _ptr(a[1]), _ptr(a[2]), _ptr(r), layout))

    def initialize(self):
        """``initialize!(s)`` (src/FluidFlowSimulation.jl:67-91)."""
        self._check(self._L.ffs_initialize(self._h))

    def advance_in_time(self, nsteps: int = 1):
        """``advance_in_time!(s)`` repeated ``nsteps`` times (src/models.jl:3-17)."""
        self._check(self._L.ffs_step(self._h, int(nsteps)))

    def finalize(self):
        """The tail of ``run_simulation`` after its time loop (src/FluidFlowSimulation.jl:46-49):
        ``calculate_rhs!``, the forcing and ``writestats`` at the current iteration (one
        Stats record whatever the iteration; fields, iteration and time unchanged)."""
        self._check(self._L.ffs_finalize(self._h))

    @property
    def forcing_shells(self) -> int:
        """2D shells of the kz = 0 plane forcing (0 without it)."""
        return int(self._L.ffs_forcing_shells(self._h))

    def forcing_array(self, which: str, values=None) -> np.ndarray:
        """Per-shell state of the kz = 0 plane forcing: "R" (the ODE state of the R.N files),
        "Em" (target spectrum), "avgK" (mean wavenumber, read only), "N" (nRf/cNRf: the
        plane's non-linear transfer, the N.N files) or "Ef" (the shell energy of the last
        forcing call, read only, the Eh.N files). aForcing: "R" is its (nx/2+1) x ny mode
        matrix. With values, set it."""
        if self.params.plane_forcing == 6:   # aForcing: R per mode
            if which != "R":
                raise ValueError("aForcing keeps only R (per mode)")
            nxh = self.nx // 2 + 1
            a = (np.zeros(nxh * self.ny) if values is None
                 else np.ascontiguousarray(np.asarray(values, dtype=np.float64).reshape(self.ny, nxh)).reshape(-1))
            self._check(self._L.ffs_forcing_array(self._h, 5, a.ctypes.data_as(_D), a.size,
                                                  0 if values is None else 1))
            return a.reshape(self.ny, nxh).T.copy()   # the reference's R[i, j]: kx rows, y columns
        w = {"R": 0, "Em": 1, "avgK": 2, "N": 3, "Ef": 4}[which]
        n = self.forcing_shells
        a = np.zeros(n) if values is None else np.ascontiguousarray(values, dtype=np.float64)
        self._check(self._L.ffs_forcing_array(self._h, w, a.ctypes.data_as(_D), n, 0 if values is None else 1))
        return a

    OUTPUT_FIELDS = ("T11", "T12", "T13", "T22", "T23", "cs", "cp", "dflux1", "dflux2", "dflux3")

    def capture_output(self, on: bool = True) -> None:
        """Capture writeoutput's LES fields (T11..T23, cs, cp, dflux1..3; src/output.jl:22-42)
        at every output step and at the run's tail."""
        self._check(self._L.ffs_capture_output(self._h, 1 if on else 0))

    def output_fields(self) -> tuple[int, dict]:
        """The fields of the most recent capture that this configuration has, by the
        reference's file stem, and the iteration they belong to."""
        out, it = {}, c_int64(-1)
        for i, name in enumerate(self.OUTPUT_FIELDS):
            a = np.empty((self.nz, self.ny, self.nx))
            rc = self._L.ffs_output_field(self._h, i, a.ctypes.data_as(_D), ctypes.byref(it))
            if rc == -1:     # FFS_EINVAL: not a field of this configuration
                continue
            self._check(rc)
            out[name] = a
        return it.value, out

    def fields(self, layout: int = 0):
        shape = (self.nz, self.ny, self.nx if layout == 0 else 2 * (self.nx // 2 + 1))
        out = [np.empty(shape) for _ in range(4 if self.has_density else 3)]
        rho = out[3] if self.has_density else None
        self._check(self._L.ffs_get_fields(self._h, _ptr(out[0]), _ptr(out[1]), _ptr(out[2]), _ptr(rho), layout))
        return tuple(out)

    def spectral(self, comp: int) -> np.ndarray:
        out = np.empty((self.nz, self.ny, self.nx // 2 + 1), dtype=np.complex128)
        self._check(self._L.ffs_get_spectral(self._h, comp, out.ctypes.data_as(_D)))
        return out

    def set_spectral(self, comp: int, a: np.ndarray):
        a = np.ascontiguousarray(a, dtype=np.complex128)
        self._check(self._L.ffs_set_spectral(self._h, comp, a.ctypes.data_as(_D)))

    def records(self) -> np.ndarray:
        """Pending stats records, drained by the read: the Stats.txt columns, 13 Scales.txt
        inputs, then with specFil the Stats_fil.txt columns (``stats_fil_rows``)."""
        n = self._L.ffs_stats_records(self._h, None, 0)
        out = np.empty((max(n, 0), self.rec_ncols))
        if n > 0:
            self._L.ffs_stats_records(self._h, out.ctypes.data_as(_D), n)
        return out

    def stats_rows(self) -> np.ndarray:
        return self.records()[:, : self.ncols]

    @property
    def has_stats_fil(self) -> bool:
        """specFil != 0: every record also carries the Stats_fil.txt row (stats.jl:48-52)."""
        return self.rec_ncols > self.ncols + 13

    def stats_fil_rows(self, records: np.ndarray | None = None) -> np.ndarray:
        """Stats_fil.txt rows (iteration, time, then the filtered columns) of records."""
        r = self.records() if records is None else records
        o = self.ncols + 13
        return np.concatenate([r[:, :2], r[:, o:o + self.ncols - 2]], axis=1)

    def stats(self) -> np.ndarray:
        """The Stats.txt row of the most recent stats iteration (``ffs_stats``); pending
        records stay available to ``records``/``stats_rows``."""
        out = np.empty(self.ncols)
        self._check(self._L.ffs_stats(self._h, out.ctypes.data_as(_D), self.ncols))
        return out

    def spectrum(self) -> tuple[np.ndarray, np.ndarray]:
        """u spectrum of the current state (``ffs_spectrum``): the reference's u.specH on
        the horizontal bins and u_h.specV + u_v.specV on the vertical bins."""
        H, V = np.empty(self.lenH), np.empty(self.lenV)
        self._check(self._L.ffs_spectrum(self._h, H.ctypes.data_as(_D), V.ctypes.data_as(_D), self.lenH, self.lenV))
        return H, V

    def scales_numbers(self, records: np.ndarray) -> tuple[list[list[float]], list[list[float]]]:
        """Scales.txt and Numbers.txt rows (with iteration and time) of drained records."""
        p = self.params
        names = self.header.split(",")
        n2 = p.gravity * p.density_gradient if (p.density and p.gravity_dir == 2) else 0.0
        sc, nu = [], []
        for r in records:
            a, b = _scales.scales_numbers(r, names, self.ncols, p.nu, p.lx, p.ly, p.lz, bool(p.density), n2)
            sc.append([r[0], r[1]] + a)
            nu.append([r[0], r[1]] + b)
        return sc, nu

    @property
    def spectrum_fields(self) -> list[str]:
        buf = ctypes.create_string_buffer(1024)
        n = self._L.ffs_spectrum_fields(self._h, buf, len(buf))   # the field count, or an error code
        if n < 0:
            self._check(n)
        return buf.value.decode().split(",")

    def spectra(self) -> list[dict]:
        """Pending spectrum records as {"iteration", "<field>.specH", "<field>.specV", ...},
        plus the h + v totals "<name>.specH" of writespectrum (spec.jl:173-194)."""
        names = self.spectrum_fields
        H, V = self.lenH, self.lenV
        rl = 1 + len(names) * (H + V)
        n = self._L.ffs_spectrum_records(self._h, None, 0)
        out = np.empty((max(n, 0), rl))
        if n > 0:
            self._L.ffs_spectrum_records(self._h, out.ctypes.data_as(_D), n)
        res = []
        for r in out:
            rec = {"iteration": int(r[0])}
            for i, nm in enumerate(names):
                o = 1 + i * (H + V)
                rec[f"{nm}.specH"] = r[o:o + H]
                rec[f"{nm}.specV"] = r[o + H:o + H + V]
            for base in ("u", "vis", "nl", "press", "les", "hvis", "u_fil", "vis_fil", "nl_fil", "press_fil",
                         "hvis_fil"):
                if f"{base}_h.specH" in rec:
                    rec[f"{base}.specH"] = rec[f"{base}_h.specH"] + rec[f"{base}_v.specH"]
            res.append(rec)
        return res

    @property
    def iteration(self) -> int:
        return int(self._L.ffs_iteration(self._h))

    @property
    def time(self) -> float:
        return float(self._L.ffs_time(self._h))

    @property
    def dt(self) -> float:
        return float(self._L.ffs_dt(self._h))

    # ---------------------------------------------------------------- timing
    def time_steps(self, nsteps: int) -> float:
        ms = c_double()
        self._check(self._L.ffs_time_steps(self._h, int(nsteps), byref(ms)))
        return ms.value

    def profile_kernels(self, nsteps: int) -> dict[str, float]:
        names = ctypes.create_string_buffer(1024)
        ms = (c_double * 16)()
        nk = c_int32()
        self._check(self._L.ffs_profile_kernels(self._h, int(nsteps), names, 1024, ms, 16, byref(nk)))
        keys = names.value.decode().split(",")
        return {k: ms[i] for i, k in enumerate(keys[: nk.value])}

    @property
    def launches_per_step(self) -> int:
        return int(self._L.ffs_launches_per_step(self._h))

    @property
    def tuning(self) -> str:
        """Launch shapes picked by the autotuner and the candidates' timings ('' if off)."""
        buf = ctypes.create_string_buffer(8192)
        self._check(self._L.ffs_tuning_report(self._h, buf, len(buf)))
        return buf.value.decode()

    @property
    def device_bytes(self) -> int:
        return int(self._L.ffs_device_bytes(self._h))

    @property
    def stream(self) -> int:
        return int(self._L.ffs_stream(self._h) or 0)


# ----------------------------------------------------------------------------------
# Reference output formats
# ----------------------------------------------------------------------------------

def stats_line(row) -> str:
    """One Stats.txt row (``join(file,(init,time,results...,"\\n"),",","")``, stats.jl:44-46)."""
    return ",".join([str(int(row[0]))] + [julia_float(v) for v in row[1:]]) + "\n"


def write_spectrum_files(folder: Path, rec: dict, KH: np.ndarray, KRZ: np.ndarray, rhosource: float | None = None,
                         tail: bool = False) -> None:
    """``write_spec`` (spec.jl:1-146, 173-194): tab-separated (k, E) pairs per spectrum
    file. rhosource = -drho/dz / g_z turns the buoyancy spectra into rhosource.*. The
    forcing spectrum forcing_h.* comes from advance_in_time! (models.jl:6-9), so the run's
    tail (tail=True) writes none."""
    i = rec["iteration"]

    def put(name, k, e):
        with open(folder / f"{name}.{i}", "w") as f:
            for a, b in zip(k, e):
                f.write(f"{julia_float(float(a))}\t{julia_float(float(b))}\n")

    for key, e in rec.items():
        if key == "iteration" or (tail and key.startswith("forcing_h.")):
            continue
        put(key, KH if key.endswith("specH") else KRZ, e)
    if rhosource is not None and "buoyancy_v.specH" in rec:
        put("rhosource.specH", KH, rec["buoyancy_v.specH"] * rhosource)
        put("rhosource.specV", KRZ, rec["buoyancy_v.specV"] * rhosource)
    if rhosource is not None and "buoyancy_fil_v.specH" in rec:   # spec.jl:85-95
        put("rhosource_fil.specH", KH, rec["buoyancy_fil_v.specH"] * rhosource)
        put("rhosource_fil.specV", KRZ, rec["buoyancy_fil_v.specV"] * rhosource)


def run_simulation(folder: str | Path = ".", precision: str | None = None, device: int = 0) -> Simulation:
    """Mirror of ``run_simulation()`` (src/FluidFlowSimulation.jl:23-65) on the GPU engine."""
    folder = Path(folder)
    d = readglobal(folder / "global")
    sim = Simulation.from_global(d, precision=precision, device=device)
    p = sim.params
    start = int(p.start)
    u = [_fields.read_field(folder / f"u{i}.{start}", p.nx, p.ny, p.nz) for i in (1, 2, 3)]
    rho = None   # rho.$start (density_stratification_types.jl:166) or scalar.$start (simulationtypes.jl:325)
    if sim.has_density and (folder / f"{sim.scalar_name}.{start}").exists():
        rho = _fields.read_field(folder / f"{sim.scalar_name}.{start}", p.nx, p.ny, p.nz)
    sim.set_fields(*u, rho)
    total = int(d["nt"]) if "nt" in d else (1 << 62) - start
    lengthtime = float(d["timeDuration"]) if "timeDuration" in d else float("inf")
    if start == 0:   # writeheader (stats.jl:9-37)
        (folder / "Stats.txt").write_text(sim.header + "\n")
        if sim.has_stats_fil:
            (folder / "Stats_fil.txt").write_text(sim.header + "\n")
        (folder / "Scales.txt").write_text(_scales.scales_header(bool(p.density)) + "\n")
        (folder / "Numbers.txt").write_text(_scales.numbers_header(bool(p.density)) + "\n")
    sim.initialize()
    if sim.params.les:
        sim.capture_output(True)    # T11..T23, cs, cp, dflux of each output step
    if p.plane_forcing == 6 and (folder / f"R.{start}").exists():   # initialize!(f::AForcing), forcing_types.jl:108-113
        rm = np.loadtxt(folder / f"R.{start}", ndmin=2)
        sim.forcing_array("R", rm.reshape(p.nx // 2 + 1, p.ny).T)
    if sim.forcing_shells:
        # initialize!(f::RfForcing) (forcing_types.jl:66-73): the target spectrum from
        # targSpectrum.dat when present (calculate_Em!, linear interpolation at avgK), else
        # the initial field's; R from R.$start when present
        tf = folder / "targSpectrum.dat"
        if p.plane_forcing != 3 and tf.exists():
            data = np.loadtxt(tf, skiprows=1)
            sim.forcing_array("Em", np.interp(sim.forcing_array("avgK"), data[:, 0], data[:, 1]))
        rf = folder / f"R.{start}"
        if rf.exists():
            sim.forcing_array("R", np.loadtxt(rf).reshape(-1))
        nf = folder / f"N.{start}"   # nRfForcing / cNRfForcing (forcing_types.jl:114-116)
        if p.plane_forcing in (4, 5) and nf.exists():
            sim.forcing_array("N", np.loadtxt(nf).reshape(-1))
    final_step = start + total
    final_time = p.start_time + lengthtime
    kx1, ky1 = 1.0 / p.lx, 1.0 / p.ly
    KH = (np.arange(p.nx // 2 + 1) / p.lx) if kx1 >= ky1 else (np.arange(p.ny // 2 + 1) / p.ly)
    KRZ = np.arange(p.nz // 2 + 1) / p.lz
    wt = int(p.write_time)
    # rhosource = -(buoyancy / g_z) * drho/dz (spec.jl:53-54)
    rhos = (-p.density_gradient / p.gravity) if (p.density and p.gravity_dir == 2 and p.gravity != 0) else None

    def flush(tail=False):
        recs = sim.records()
        with open(folder / "Stats.txt", "a") as f:
            for r in recs[:, : sim.ncols]:
                f.write(stats_line(r))
        if sim.has_stats_fil:
            with open(folder / "Stats_fil.txt", "a") as f:
                for r in sim.stats_fil_rows(recs):
                    f.write(stats_line(r))
        sc, nums = sim.scales_numbers(recs)
        for name, rows in (("Scales.txt", sc), ("Numbers.txt", nums)):
            with open(folder / name, "a") as f:
                for r in rows:
                    f.write(stats_line(r))
        for rec in sim.spectra():
            write_spectrum_files(folder, rec, KH, KRZ, rhos, tail=tail)

    steps = 0
    les_pending = None   # the output iteration whose LES fields the next step captures
    while sim.iteration < final_step and sim.time < final_time:     # FluidFlowSimulation.jl:42-44
        it = sim.iteration
        nxt = min(final_step, (it // wt + 1) * wt)
        if lengthtime != float("inf"):
            nxt = it + 1       # time-limited runs check the clock every step
        sim.advance_in_time(nxt - it)
        steps += nxt - it
        flush()
        if les_pending is not None:
            _write_les_output(folder, sim, les_pending)
            les_pending = None
        # the reference writes u.N from calculate_rhs! when the step from N starts
        # (is_output_time, simulationtypes.jl:102, models.jl:158); the LES fields of that
        # calculate_rhs! are captured by the step and written after it
        if sim.iteration % wt == 0 and sim.iteration < final_step and sim.time < final_time:
            _write_output(folder, sim)
            _write_forcing_output(folder, sim, sim.iteration, _forcing_state(sim))
            if sim.params.les:
                les_pending = sim.iteration
    # the tail (FluidFlowSimulation.jl:46-58): calculate_rhs!, forcing and a Stats row at the
    # final iteration. The final files come from the tail's calculate_rhs! when the iteration
    # is a multiple of writeTime (before the tail's forcing), else from the explicit
    # writeoutput after it.
    in_rhs = sim.iteration % wt == 0 and steps > 0
    pre = _forcing_state(sim) if in_rhs else None
    sim.finalize()
    flush(tail=True)
    _write_output(folder, sim)
    _write_forcing_output(folder, sim, sim.iteration, pre if in_rhs else _forcing_state(sim))
    if sim.params.les:
        _write_les_output(folder, sim, sim.iteration)
    if p.plane_forcing == 1:   # writedlm("R.$(iteration)", R) for rfForcing (FluidFlowSimulation.jl:60-62)
        write_dlm(folder / f"R.{sim.iteration}", sim.forcing_array("R"))
    return sim


def _write_output(folder: Path, sim: Simulation) -> None:
    """``writeoutput`` (src/output.jl:1-30): u1.N u2.N u3.N (+ rho.N or scalar.N)."""
    f = sim.fields()
    i = sim.iteration
    for k in range(3):
        _fields.write_field(folder / f"u{k + 1}.{i}", f[k])
    if sim.has_density:
        _fields.write_field(folder / f"{sim.scalar_name}.{i}", f[3])


def write_dlm(path: Path, rows) -> None:
    """``writedlm`` with its default tab delimiter: one line per value of a vector, per
    tuple of an iterator of tuples, per row of a matrix; values printed as Julia prints them."""
    a = np.asarray(rows, dtype=np.float64)
    with open(path, "w") as f:
        for r in (a if a.ndim == 2 else a[:, None]):
            f.write("\t".join(julia_float(float(v)) for v in r) + "\n")


def _forcing_state(sim: Simulation) -> dict:
    """The kz = 0 forcing arrays writeoutput writes (output.jl:45-67): R, and Eh = (avgK, Ef)
    and N by kind."""
    kind = int(sim.params.plane_forcing)
    if kind == 6:                                       # aForcing: R (per mode)
        return {"R": sim.forcing_array("R")}
    if kind in (1, 2, 4, 5):                            # rf, cRf, nRf, cNRf
        st = {"R": sim.forcing_array("R"), "Eh": np.stack([sim.forcing_array("avgK"), sim.forcing_array("Ef")], 1)}
        if kind in (4, 5):
            st["N"] = sim.forcing_array("N")
        return st
    return {}


def _write_forcing_output(folder: Path, sim: Simulation, it: int, state: dict) -> None:
    for name, a in state.items():
        write_dlm(folder / f"{name}.{it}", a)


def _write_les_output(folder: Path, sim: Simulation, it: int) -> None:
    """writeoutput's LES fields (output.jl:22-42): T11..T23, cs (cp) and dflux1..3, captured
    by the calculate_rhs! of iteration it."""
    got, fields = sim.output_fields()
    if got != it:
        raise RuntimeError(f"LES output capture holds iteration {got}, expected {it}")
    for name, a in fields.items():
        _fields.write_field(folder / f"{name}.{it}", a)
