"""Field files and initial conditions.

Field files follow the reference: raw little-endian Float64, x fastest, the unpadded
nx*ny*nz block (``write(file, PaddedArray)`` in src/output.jl:6-8; the InplaceRealFFT
writer is not vendored, so the header-less raw format is an assumption checked by file
size). Arrays here are numpy ``[z, y, x]`` (C order), the same memory order.
"""
from __future__ import annotations

from pathlib import Path

import numpy as np


def write_field(path: str | Path, a: np.ndarray) -> None:
    np.ascontiguousarray(a, dtype="<f8").tofile(str(path))


def read_field(path: str | Path, nx: int, ny: int, nz: int) -> np.ndarray:
    p = Path(path)
    n = nx * ny * nz
    size = p.stat().st_size
    if size == 8 * n:
        return np.fromfile(str(p), dtype="<f8").reshape(nz, ny, nx)
    nrx = 2 * (nx // 2 + 1)
    if size == 8 * nrx * ny * nz:   # padded block
        return np.fromfile(str(p), dtype="<f8").reshape(nz, ny, nrx)[:, :, :nx].copy()
    raise ValueError(f"{p}: {size} bytes is neither {8 * n} (nx*ny*nz Float64) nor the padded size")


def taylor_green(n: int) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """README.md:12-20: u1 = cos x sin y sin z, u2 = -sin x cos y sin z, u3 = 0 on x_i = 2 pi i / n."""
    x = 2 * np.pi * np.arange(n) / n
    X, Y, Z = x[None, None, :], x[None, :, None], x[:, None, None]
    u1 = np.cos(X) * np.sin(Y) * np.sin(Z)
    u2 = -np.sin(X) * np.cos(Y) * np.sin(Z)
    return u1, u2, np.zeros((n, n, n))


def random_spectrum(n: int, k0: float, seed: int, urms: float = 1.0, cutoff: float = 2.0 / 3.0,
                    L: float = 1.0) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """Seeded random-phase, divergence-free field with E(k) ~ k^4 exp(-2 (k/k0)^2).

    For the retained (dealiased) modes with |k| > 0: u_hat = A(|k|) * (complex Gaussian
    projected perpendicular to k), A^2 = E(k) / (4 pi k^2). The half spectrum is brought
    to physical space (which makes it Hermitian), projected again and scaled so that
    sqrt(<u.u>/3) = urms. Deterministic for a given seed (numpy PCG64).
    """
    rng = np.random.default_rng(seed)
    nxh = n // 2 + 1
    kx = np.arange(nxh) / L
    ky = np.fft.fftfreq(n, 1.0 / n) / L
    KX, KY, KZ = kx[None, None, :], ky[None, :, None], ky[:, None, None]
    K2 = KX ** 2 + KY ** 2 + KZ ** 2
    kmax = (n // 2) / L
    c = (cutoff * kmax) ** 2
    keep = (KX ** 2 <= c) & (KY ** 2 <= c) & (KZ ** 2 <= c) & (K2 > 0)
    g = rng.standard_normal((3, n, n, nxh)) + 1j * rng.standard_normal((3, n, n, nxh))
    with np.errstate(divide="ignore", invalid="ignore"):
        kd = (KX * g[0] + KY * g[1] + KZ * g[2]) / K2
        g = np.stack([g[0] - kd * KX, g[1] - kd * KY, g[2] - kd * KZ])
        k = np.sqrt(K2)
        E = k ** 4 * np.exp(-2.0 * (k / k0) ** 2)
        A = np.sqrt(E / (4 * np.pi * K2))
    A = np.where(keep, A, 0.0)
    uh = np.nan_to_num(g) * A[None]
    u = np.fft.irfftn(uh, s=(n, n, n), axes=(1, 2, 3))
    # project the (Hermitian) field once more and normalise
    uh = np.fft.rfftn(u, axes=(1, 2, 3))
    with np.errstate(divide="ignore", invalid="ignore"):
        kd = (KX * uh[0] + KY * uh[1] + KZ * uh[2]) / K2
    kd = np.nan_to_num(kd)
    uh = np.stack([uh[0] - kd * KX, uh[1] - kd * KY, uh[2] - kd * KZ])
    uh[:, ~keep] = 0.0
    u = np.fft.irfftn(uh, s=(n, n, n), axes=(1, 2, 3))
    s = np.sqrt(np.mean(u[0] ** 2 + u[1] ** 2 + u[2] ** 2) / 3.0)
    u = u * (urms / s)
    return u[0].copy(), u[1].copy(), u[2].copy()


def random_spectrum_modes(n: int, k0: float, seed: int, kc: int, urms: float = 1.0, L: float = 1.0):
    """Spectral form of ``random_spectrum`` for grids too large to build on the host in
    physical space: the same E(k) ~ k^4 exp(-2 (k/k0)^2), divergence-free random-phase
    field, generated directly as half-spectrum coefficients on the low-mode box
    |kx|, |ky|, |kz| <= kc (E(k) is negligible beyond ~4 k0), Hermitian on the kx = 0
    plane, scaled so that sqrt(<u.u>/3) = urms by Parseval. Returns the box
    [3][2kc+1 (kz = -kc..kc)][2kc+1 (ky)][kc+1 (kx)]; ``embed_half_spectrum`` places one
    component into the [nz][ny][nx/2+1] layout of ``Simulation.set_spectral``."""
    rng = np.random.default_rng(seed)
    m = np.arange(-kc, kc + 1) / L
    kx = np.arange(kc + 1) / L
    KX, KY, KZ = kx[None, None, :], m[None, :, None], m[:, None, None]
    K2 = KX ** 2 + KY ** 2 + KZ ** 2
    g = rng.standard_normal((3,) + K2.shape) + 1j * rng.standard_normal((3,) + K2.shape)
    with np.errstate(divide="ignore", invalid="ignore"):
        kd = (KX * g[0] + KY * g[1] + KZ * g[2]) / K2
        g = np.stack([g[0] - kd * KX, g[1] - kd * KY, g[2] - kd * KZ])
        k = np.sqrt(K2)
        A = np.sqrt(k ** 4 * np.exp(-2.0 * (k / k0) ** 2) / (4 * np.pi * K2))
    uh = np.nan_to_num(g) * np.where(K2 > 0, A, 0.0)[None]
    # Hermitian kx = 0 plane: u(0, -ky, -kz) = conj u(0, ky, kz)
    p0 = uh[:, :, :, 0]
    uh[:, :, :, 0] = 0.5 * (p0 + np.conj(p0[:, ::-1, ::-1]))
    w = np.where(np.arange(kc + 1) > 0, 2.0, 1.0)[None, None, None, :]
    e = float(np.sum(w * np.abs(uh) ** 2))   # <u.u> by Parseval
    return uh * (urms * np.sqrt(3.0 / e))


def embed_half_spectrum(box: np.ndarray, n: int, kc: int) -> np.ndarray:
    """One component of ``random_spectrum_modes`` in the [n][n][n/2+1] half-spectrum layout."""
    out = np.zeros((n, n, n // 2 + 1), dtype=np.complex128)
    idx = np.r_[np.arange(0, kc + 1), np.arange(n - kc, n)]        # fftfreq order of -kc..kc
    src = np.r_[np.arange(kc, 2 * kc + 1), np.arange(0, kc)]
    out[np.ix_(idx, idx, np.arange(kc + 1))] = box[np.ix_(src, src, np.arange(kc + 1))]
    return out
