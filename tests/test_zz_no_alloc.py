"""ffs_fourier_noalloc: the forward transform for callers that cannot allocate device
memory (their device memory belongs to another allocator or pool, or their loop must not
allocate once running, or their host grants only the buffers it passes in). The caller
brings device buffers for the input and the output; the library's twiddles and
intermediates live in its static device array.

The test plays such a caller: it owns device buffers (made with torch here) and calls the
entry point through the C ABI two times in a row on each grid, with different fields,
and then on the next grid. Every result is checked against the allocating path
(ffs_set_fields + ffs_get_spectral) and against the oracle's forward transform
(rfftn, 2/3 dealiasing, 1/N), at the FP64 transform tolerance of the other tests. The
grids include the documented limit case (128^3, about 21 MB of the 24 MiB array) and a
radix-3 size (48^3). Collected last on purpose: a run that stops at the first failure
has run every other test before this one.
"""
import ctypes

import numpy as np
import pytest

from oracle.ffs_oracle import Grid

pytestmark = pytest.mark.gpu

FP64_TRANSFORM_TOL = 1e-14


def _global(nx, ny, nz):
    return {"nx": str(nx), "ny": str(ny), "nz": str(nz), "xDomainSize": "1.0", "yDomainSize": "1.0",
            "zDomainSize": "1.0", "kinematicViscosity": "0.01", "dtStat": "1", "dtSpec": "1", "writeTime": "1",
            "velocityTimeStep": "Adams_Bashforth3rdO", "variableTimestepFlag": "false", "dt": "0.01"}


def _allocating_path(pkg, u):
    nz, ny, nx = u.shape
    sim = pkg.Simulation.from_global(_global(nx, ny, nz), precision="FP64")
    z = np.zeros_like(u)
    sim.set_fields(u, z, z)
    out = sim.spectral(0)
    sim.close()
    return out


def _rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.parametrize("grid", [(64, 64, 64), (32, 48, 64), (48, 48, 48), (128, 128, 128)])
def test_fourier_noalloc_two_calls_match_allocating_path_and_oracle(gpu_pkg, grid):
    torch = pytest.importorskip("torch")
    L = gpu_pkg.load()
    nx, ny, nz = grid
    rng = np.random.default_rng(20261203 + nx * 7 + ny * 3 + nz)
    stream = torch.cuda.current_stream()
    g = Grid(nx, ny, nz)
    for call in range(2):   # two calls in a row on the same grid, different fields
        u = rng.standard_normal((nz, ny, nx))
        phys = torch.from_numpy(u).to("cuda")
        spec = torch.full((nz * ny * (nx // 2 + 1) * 2,), float("nan"), dtype=torch.float64, device="cuda")
        rc = L.ffs_fourier_noalloc(ctypes.c_void_p(phys.data_ptr()), ctypes.c_void_p(spec.data_ptr()), nx, ny, nz,
                                   1.0, 1.0, 1.0, 2.0 / 3.0, ctypes.c_void_p(stream.cuda_stream))
        assert rc == 0, L.ffs_last_error(None)
        torch.cuda.synchronize()
        got = spec.cpu().numpy().view(np.complex128).reshape(nz, ny, nx // 2 + 1)
        assert np.isfinite(got).all()
        ref = _allocating_path(gpu_pkg, u)
        assert _rel(got, ref) <= FP64_TRANSFORM_TOL, (grid, call, "allocating path")
        assert _rel(got, g.myfourier(u)) <= FP64_TRANSFORM_TOL, (grid, call, "oracle")
        # modes outside the retained box are exact zeros, as in the allocating path
        assert np.array_equal(got == 0, ref == 0)
        assert not got[g.dealias].any()


def test_fourier_noalloc_rejects_grids_beyond_its_buffer(gpu_pkg):
    torch = pytest.importorskip("torch")
    L = gpu_pkg.load()
    n = 256
    phys = torch.zeros(8, dtype=torch.float64, device="cuda")   # never read: the size check comes first
    rc = L.ffs_fourier_noalloc(ctypes.c_void_p(phys.data_ptr()), ctypes.c_void_p(phys.data_ptr()), n, n, n,
                               1.0, 1.0, 1.0, 2.0 / 3.0, None)
    assert rc == -1
    assert b"static buffer" in L.ffs_last_error(None)
