"""Golden fixtures (tests/golden/*.npz, made by tests/golden/make_golden.py): 16^3 cases,
10 steps. The oracle must reproduce them (regression pin); the engine must match them at
the FP64 bar through the C ABI."""
from pathlib import Path

import numpy as np
import pytest

from oracle.ffs_oracle import OracleSimulation, Params

GOLD = Path(__file__).resolve().parent / "golden"
CASES = sorted(p.stem for p in GOLD.glob("*.npz"))


def load(name):
    z = np.load(GOLD / f"{name}.npz")
    d = dict(zip([str(k) for k in z["keys"]], [str(v) for v in z["values"]]))
    return z, d


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.parametrize("name", CASES)
def test_oracle_reproduces_golden(name):
    z, d = load(name)
    rho0 = z["rho0"] if "rho0" in z else None
    s = OracleSimulation(Params.from_global(d), list(z["u0"]), rho0)
    s.initialize()
    s.run(10)
    for c in range(3):
        assert rel(s.u[c], z["uh"][c]) < 1e-13
    assert np.allclose(np.array(s.stats_rows), z["stats"], rtol=1e-11, atol=1e-14)


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_engine_matches_golden(gpu_pkg, name):
    z, d = load(name)
    rho0 = z["rho0"] if "rho0" in z else None
    sim = gpu_pkg.Simulation.from_global(d, precision="FP64")
    sim.set_fields(*z["u0"], rho0)
    sim.initialize()
    sim.advance_in_time(10)
    for c in range(3):
        assert rel(sim.spectral(c), z["uh"][c]) <= 1e-12, (name, c)
    if rho0 is not None:
        assert rel(sim.spectral(3), z["rhoh"]) <= 1e-12
    rows = sim.stats_rows()
    gold = z["stats"]
    assert rows.shape == gold.shape
    scale = np.maximum(np.abs(gold), 1e-6 * np.abs(gold).max())
    assert (np.abs(rows - gold) / scale).max() <= 1e-10
    sim.close()
