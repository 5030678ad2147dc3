"""ffs_fourier_noalloc: the forward transform for callers that cannot allocate device memory
(code inside a CUDA stream capture, memory owned by another allocator or pool, hosts
that forbid allocations at run time). The caller brings device buffers for the input and
the output; the library's intermediates live in its static device array.

The test plays such a caller: it owns device buffers (made with torch here), calls the
entry point through the C ABI twice in a row with different fields and grids, and checks
each result against the allocating path (ffs_set_fields + ffs_get_spectral) at the FP64
transform tolerance of the other tests. Collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

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


def test_fourier_noalloc_matches_allocating_path(gpu_pkg):
    torch = pytest.importorskip("torch")
    L = gpu_pkg.load()
    rng = np.random.default_rng(20261203)
    stream = torch.cuda.current_stream()
    for (nx, ny, nz) in ((64, 64, 64), (32, 48, 64)):
        u = rng.standard_normal((nz, ny, nx))
        phys = torch.from_numpy(u).to("cuda")
        spec = torch.full((nz * ny * (nx // 2 + 1) * 2,), float("nan"), dtype=torch.float64, device="cuda")
        rc = L.ffs_fourier_noalloc(ctypes.c_void_p(phys.data_ptr()), ctypes.c_void_p(spec.data_ptr()), nx, ny, nz,
                                   1.0, 1.0, 1.0, 2.0 / 3.0, ctypes.c_void_p(stream.cuda_stream))
        assert rc == 0, L.ffs_last_error(None)
        torch.cuda.synchronize()
        got = spec.cpu().numpy().view(np.complex128).reshape(nz, ny, nx // 2 + 1)
        ref = _allocating_path(gpu_pkg, u)
        assert np.isfinite(got).all()
        err = np.linalg.norm(got - ref) / np.linalg.norm(ref)
        assert err <= FP64_TRANSFORM_TOL, ((nx, ny, nz), err)
        # modes outside the retained box are exact zeros, as in the allocating path
        assert np.array_equal(got == 0, ref == 0)


def test_fourier_noalloc_rejects_grids_beyond_its_buffer(gpu_pkg):
    torch = pytest.importorskip("torch")
    L = gpu_pkg.load()
    n = 256
    phys = torch.zeros(8, dtype=torch.float64, device="cuda")   # never read: the size check comes first
    rc = L.ffs_fourier_noalloc(ctypes.c_void_p(phys.data_ptr()), ctypes.c_void_p(phys.data_ptr()), n, n, n,
                               1.0, 1.0, 1.0, 2.0 / 3.0, None)
    assert rc == -1
    assert b"static buffer" in L.ffs_last_error(None)
