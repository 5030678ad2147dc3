"""Regenerate the full-run fixture of the Taylor-Green 64^3 configuration.

The configuration: u1 = cos x sin y sin z, u2 = -sin x cos y sin z, u3 = 0 on the 64^3
grid x_i = 2 pi i / 64 (README.md:12-20 of the reference), nu = 0.0333333, dt = 0.05,
500 steps, 2/3 dealiasing, no forcing, no LES, stats every 20 steps. It runs on ETD3
(the reference's default integrator): with AB3 the viscous term is explicit and
nu k_max^2 dt = 0.0333333 * 3 * 21^2 * 0.05 = 2.2 lies far outside AB3's stability
interval, so that run blows up within ~40 steps (tests/test_oracle_kat.py checks this).

The FP64 oracle runs the whole configuration, then the tail of run_simulation
(FluidFlowSimulation.jl:46-49). Stored: the `global` keys, the Stats/Scales/Numbers rows
(25 rows from the loop at iterations 0, 20, ..., 480, then the tail's row at 500), and
the final spectral state on the box |k_i| <= 8 with the per-component L2 norms of the
whole final state.

    python tests/golden/make_config_golden.py
"""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle.ffs_oracle import OracleSimulation, Params, taylor_green  # noqa: E402

OUT = Path(__file__).resolve().parent / "configs"
TG64 = {"nx": "64", "ny": "64", "nz": "64", "xDomainSize": "1.0", "yDomainSize": "1.0", "zDomainSize": "1.0",
        "kinematicViscosity": "0.0333333", "dtStat": "20", "dtSpec": "1000000000", "writeTime": "1000000000",
        "velocityTimeStep": "ETD3rdO", "variableTimestepFlag": "false", "dt": "0.05", "nt": "500"}
KBOX = 8


def low_box(uh: np.ndarray, k: int) -> np.ndarray:
    """Modes |kx|, |ky|, |kz| <= k of a [comp][z][y][kx] half spectrum, as [comp][kz][ky][kx]
    with kz, ky in -k..k."""
    idx = np.r_[0:k + 1, -k:0]
    return uh[:, idx][:, :, idx][:, :, :, : k + 1]


def main():
    OUT.mkdir(exist_ok=True)
    s = OracleSimulation(Params.from_global(TG64), taylor_green(64))
    s.initialize()
    s.run(int(TG64["nt"]))
    s.finalize()
    np.savez_compressed(OUT / "tg64_etd3_500.npz", keys=np.array(list(TG64.keys())),
                        values=np.array(list(TG64.values())), stats=np.array(s.stats_rows),
                        scales=np.array(s.scales_rows), numbers=np.array(s.numbers_rows),
                        ubox=low_box(s.u, KBOX), unorm=np.array([np.linalg.norm(s.u[c]) for c in range(3)]),
                        kbox=np.array(KBOX))
    print("tg64", s.iteration, s.time, len(s.stats_rows))


if __name__ == "__main__":
    main()
