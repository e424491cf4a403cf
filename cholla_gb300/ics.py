"""Seeded initial conditions for the benchmark and test problems (numpy, host side).

The reference has no random-field initial condition, so these generators are new: a
lognormal density and k^-2 velocity fields for the turbulence-like hydro box, a curl of a
k^-3 vector potential for MHD (spectra summed over shells of |k|), the Sod tube, and the Sedov-like blasts and rotated Sod
tubes of the serving workload.  `linear_wave` restates the reference's Linear_Wave initial
condition, on which its system tests measure the scheme's error.  Every array is field-major [f, z, y, x] with ghost cells,
matching U[f*n_cells + x + y*nx + z*nx*ny].
"""
from __future__ import annotations

import math

import numpy as np


def n_fields(dual_energy: bool, mhd: bool = False, n_scalars: int = 0) -> int:
    return 5 + n_scalars + (3 if mhd else 0) + (1 if dual_energy else 0)


try:  # multi-threaded FFTs where scipy is present (same transform as numpy's, to rounding)
    import scipy.fft as _fft

    def _rfftn(a):
        return _fft.rfftn(a, workers=-1, overwrite_x=True)

    def _irfftn(a, n):
        return _fft.irfftn(a, s=(n, n, n), workers=-1, overwrite_x=True)
except ImportError:  # pragma: no cover
    def _rfftn(a):
        return np.fft.rfftn(a)

    def _irfftn(a, n):
        return np.fft.irfftn(a, s=(n, n, n), axes=(0, 1, 2))

_AMP: dict = {}


def _spectral_amplitude(n: int, slope: float) -> np.ndarray:
    key = (n, slope)
    if key not in _AMP:
        k = np.fft.fftfreq(n) * n
        kr = np.fft.rfftfreq(n) * n
        kk = np.sqrt(k[:, None, None] ** 2 + k[None, :, None] ** 2 + kr[None, None, :] ** 2)
        amp = np.zeros_like(kk)
        nz = kk > 0
        amp[nz] = kk[nz] ** ((slope - 2.0) / 2.0)
        _AMP.clear()
        _AMP[key] = amp
    return _AMP[key]


def gaussian_random_field(n: int, slope: float, rng: np.random.Generator) -> np.ndarray:
    """Periodic unit-variance Gaussian random field on n^3 cells whose spectrum, summed over
    shells of |k| (the turbulence convention, E(k) dk), goes as k^slope: Fourier amplitudes
    |f_k| ~ k^((slope - 2) / 2).  (A k^-2 slope is Burgers-like: smooth at the grid scale.  With
    the slope put on |f_k|^2 instead, a k^-2 field is white at the grid scale, with Mach-2 jumps
    between neighbouring cells from which even the exact FP64 scheme fails within a few steps.)"""
    amp = _spectral_amplitude(n, slope)
    spec = _rfftn(rng.standard_normal((n, n, n)))
    spec *= amp
    f = _irfftn(spec, n)
    f -= f.mean()
    f /= f.std()
    return f


def pad_periodic(real: np.ndarray, ng: int) -> np.ndarray:
    """Add ng ghost layers filled periodically to a [f, z, y, x] array of real cells."""
    return np.ascontiguousarray(np.pad(real, ((0, 0), (ng, ng), (ng, ng), (ng, ng)), mode="wrap"))


def _turbulence_box_torch(torch, n, ng, gamma, rng, sigma, mach, pressure, dual_energy):
    """turbulence_box with the transforms and the arithmetic in torch's multi-threaded CPU kernels
    (the same noise, spectrum and formulas; results agree with the numpy form to rounding)."""

    def grf(slope):
        f = torch.fft.irfftn(torch.fft.rfftn(torch.from_numpy(rng.standard_normal((n, n, n)))) *
                             torch.from_numpy(_spectral_amplitude(n, slope)), s=(n, n, n))
        f -= f.mean()
        f /= f.std(correction=0)
        return f

    g = grf(-2.0)
    rho = torch.exp(sigma * g - 0.5 * sigma * sigma)
    del g
    v = torch.stack([grf(-2.0) for _ in range(3)])
    cs = math.sqrt(gamma * pressure / 1.0)
    v2 = (v * v).sum(dim=0)
    scale = mach * cs / math.sqrt(float(v2.mean()))
    v *= scale
    v2 *= scale * scale
    nf = n_fields(dual_energy)
    U = torch.empty((1, nf, n, n, n), dtype=torch.float64)
    U[0, 0] = rho
    U[0, 1:4] = rho * v
    eint = pressure / (gamma - 1.0)
    U[0, 4] = eint + 0.5 * rho * v2
    if dual_energy:
        U[0, nf - 1] = eint
    del v, v2, rho
    out = torch.nn.functional.pad(U, (ng,) * 6, mode="circular")[0]
    return np.ascontiguousarray(out.numpy())


def turbulence_box(n: int, ng: int = 4, gamma: float = 5.0 / 3.0, seed: int = 0, sigma: float = 0.5,
                   mach: float = 2.0, pressure: float = 1.0, dual_energy: bool = True) -> np.ndarray:
    """Periodic cube of side 1: lognormal density (mean 1, sigma) from a Gaussian field with a
    k^-2 shell spectrum, three independent k^-2 velocity fields scaled to rms Mach `mach`,
    uniform pressure."""
    rng = np.random.default_rng(seed)
    if n >= 96:  # large boxes: multi-threaded transforms and arithmetic
        try:
            import torch

            return _turbulence_box_torch(torch, n, ng, gamma, rng, sigma, mach, pressure, dual_energy)
        except ImportError:  # pragma: no cover
            pass
    g = gaussian_random_field(n, -2.0, rng)
    rho = np.exp(sigma * g - 0.5 * sigma * sigma)
    v = np.stack([gaussian_random_field(n, -2.0, rng) for _ in range(3)])
    cs = math.sqrt(gamma * pressure / 1.0)
    v *= mach * cs / math.sqrt(np.mean(np.sum(v * v, axis=0)))
    nf = n_fields(dual_energy)
    U = np.empty((nf, n, n, n))
    U[0] = rho
    U[1:4] = rho * v
    eint = pressure / (gamma - 1.0)
    U[4] = eint + 0.5 * rho * np.sum(v * v, axis=0)
    if dual_energy:
        U[nf - 1] = eint
    return pad_periodic(U, ng)


def blast_box(n: int, ng: int = 4, gamma: float = 5.0 / 3.0, centre=(0.5, 0.5, 0.5), radius: float = 3.0,
              energy: float = 1.0, rho: float = 1.0, p: float = 1e-5, dual_energy: bool = True) -> np.ndarray:
    """Host copy of the serving workload's Sedov-like blast (the device version is cgb_ic_blast):
    uniform rho and p, plus thermal energy `energy` spread evenly over the cells whose centres
    lie within `radius` cells of `centre` (box coordinates, side 1).  Zero velocity."""
    dx = 1.0 / n
    c = (np.arange(n) + 0.5) * dx
    z, y, x = np.meshgrid(c, c, c, indexing="ij")
    r2 = (x - centre[0]) ** 2 + (y - centre[1]) ** 2 + (z - centre[2]) ** 2
    inside = r2 < (radius * dx) ** 2
    eint = np.full((n, n, n), p / (gamma - 1.0))
    eint[inside] += energy / (inside.sum() * dx ** 3)
    nf = n_fields(dual_energy)
    U = np.zeros((nf, n, n, n))
    U[0] = rho
    U[4] = eint
    if dual_energy:
        U[nf - 1] = eint
    return pad_periodic(U, ng)


def mhd_box(n: int, ng: int = 4, gamma: float = 5.0 / 3.0, seed: int = 0, beta: float = 1.0,
            vrms: float = 1.0) -> np.ndarray:
    """Periodic MHD cube of side 1: density 1, pressure 1, k^-2 velocity (rms vrms), face-centred
    B = discrete curl of a k^-3 vector potential (shell spectra) scaled to plasma beta, so
    div B = 0 to roundoff.
    The curl uses the stencil of Init_Magnetic_Field_With_Vector_Potential
    (src/utils/mhd_utilities.cu:22-44)."""
    rng = np.random.default_rng(seed)
    v = np.stack([gaussian_random_field(n, -2.0, rng) for _ in range(3)])
    v *= vrms / math.sqrt(np.mean(np.sum(v * v, axis=0)))
    A = np.stack([gaussian_random_field(n, -3.0, rng) for _ in range(3)])
    N = n + 2 * ng
    dx = 1.0 / n
    Ap = np.pad(A, ((0, 0), (ng, ng), (ng, ng), (ng, ng)), mode="wrap")  # [c, z, y, x]
    B = np.zeros((3, N, N, N))
    sl = (slice(1, None), slice(1, None), slice(1, None))
    Ax, Ay, Az = Ap[0], Ap[1], Ap[2]
    # Bx[id] = (Az[id]-Az[idymo])/dy - (Ay[id]-Ay[idzmo])/dz, etc.
    B[0][sl] = (Az[1:, 1:, 1:] - Az[1:, :-1, 1:]) / dx - (Ay[1:, 1:, 1:] - Ay[:-1, 1:, 1:]) / dx
    B[1][sl] = (Ax[1:, 1:, 1:] - Ax[:-1, 1:, 1:]) / dx - (Az[1:, 1:, 1:] - Az[1:, 1:, :-1]) / dx
    B[2][sl] = (Ay[1:, 1:, 1:] - Ay[1:, 1:, :-1]) / dx - (Ax[1:, 1:, 1:] - Ax[1:, :-1, 1:]) / dx
    # scale to beta = 2 p / <B^2>
    pressure = 1.0
    Bc = B[:, ng:-ng, ng:-ng, ng:-ng]
    B *= math.sqrt(2.0 * pressure / beta / np.mean(np.sum(Bc * Bc, axis=0)))
    rho = np.ones((n, n, n))
    U = np.empty((8, N, N, N))
    U[0] = pad_periodic(rho[None], ng)[0]
    U[1:4] = pad_periodic(rho * v, ng)
    U[5:8] = B
    # cell-centred B for the energy (mhd_utilities.h:205-237)
    bcx = 0.5 * (B[0] + np.roll(B[0], 1, axis=2))
    bcy = 0.5 * (B[1] + np.roll(B[1], 1, axis=1))
    bcz = 0.5 * (B[2] + np.roll(B[2], 1, axis=0))
    vv = pad_periodic(v, ng)
    U[4] = pressure / (gamma - 1.0) + 0.5 * U[0] * np.sum(vv * vv, axis=0) + 0.5 * (bcx ** 2 + bcy ** 2 + bcz ** 2)
    return np.ascontiguousarray(U)


def sod_1d(nx: int = 100, ng: int = 4, gamma: float = 1.4, dual_energy: bool = False, diaphragm: float = 0.5,
           left=(1.0, 0.0, 1.0), right=(0.125, 0.0, 0.1)) -> tuple[np.ndarray, float]:
    """Sod shock tube on [0, 1] with nx real cells; returns (U[f, x], dx)."""
    dx = 1.0 / nx
    x = (np.arange(nx + 2 * ng) - ng + 0.5) * dx
    nf = n_fields(dual_energy)
    U = np.zeros((nf, nx + 2 * ng))
    for side, mask in ((left, x < diaphragm), (right, x >= diaphragm)):
        d, v, p = side
        U[0, mask] = d
        U[1, mask] = d * v
        U[4, mask] = p / (gamma - 1.0) + 0.5 * d * v * v
        if dual_energy:
            U[nf - 1, mask] = p / (gamma - 1.0)
    return np.ascontiguousarray(U), dx


def linear_wave(nx: int, ny: int, nz: int, ng: int, dx: float, dy: float, dz: float, *, gamma: float, rho: float,
                P: float, A: float, eigen: dict, vx: float = 0.0, B=(0.0, 0.0, 0.0), pitch: float = 0.0,
                yaw: float = 0.0, wave_length: float = 1.0, mhd: bool = False, bounds=(0.0, 0.0, 0.0)) -> np.ndarray:
    """Linear wave initial condition (src/grid/initial_conditions.cpp:302-425 Grid3D::Linear_Wave):
    a background state (rho, vx, P, B) plus A * sin(k x_rot) times the right eigenvector `eigen`
    (keys rho, MomentumX/Y/Z, E, and Bx/By/Bz for MHD), along the direction rotated by pitch and
    yaw; k = 2 pi / wave_length.  Cell-centred positions x = bound + dx (i - ng) + dx / 2.  As in
    the reference, the face fields are set from the same cell-centred sine on the real cells
    only and the hydro fields on the real cells plus the first lower ghost layer; fill the ghost
    cells (periodic) before the first step.  Returns U[f, z, y, x] with ghost cells."""
    sy, cy, sp, cp = math.sin(yaw), math.cos(yaw), math.sin(pitch), math.cos(pitch)
    kw = 2.0 * math.pi / wave_length
    Nx, Ny, Nz = nx + 2 * ng, ny + 2 * ng, nz + 2 * ng
    nf = n_fields(False, mhd)
    U = np.zeros((nf, Nz, Ny, Nx))
    x = bounds[0] + dx * (np.arange(Nx) - ng) + 0.5 * dx
    y = bounds[1] + dy * (np.arange(Ny) - ng) + 0.5 * dy
    z = bounds[2] + dz * (np.arange(Nz) - ng) + 0.5 * dz
    Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
    sine = np.sin((cp * (X * cy + Y * sy) + Z * sp) * kw)
    e = {k: float(eigen.get(k, 0.0)) for k in ("rho", "MomentumX", "MomentumY", "MomentumZ", "E", "Bx", "By", "Bz")}
    if mhd:
        r = (slice(ng, Nz - ng), slice(ng, Ny - ng), slice(ng, Nx - ng))
        bx = B[0] + A * e["Bx"] * sine[r]
        by = B[1] + A * e["By"] * sine[r]
        bz = B[2] + A * e["Bz"] * sine[r]
        U[5][r] = bx * cp * cy - by * sy - bz * sp * cy
        U[6][r] = bx * cp * sy + by * cy - bz * sp * sy
        U[7][r] = bx * sp + bz * cp
    h = (slice(ng - 1, Nz - ng), slice(ng - 1, Ny - ng), slice(ng - 1, Nx - ng))
    sh = sine[h]
    U[0][h] = rho + A * e["rho"] * sh
    mx = rho * vx + A * e["MomentumX"] * sh
    my = A * e["MomentumY"] * sh
    mz = A * e["MomentumZ"] * sh
    U[1][h] = mx * cp * cy - my * sy - mz * sp * cy
    U[2][h] = mx * cp * sy + my * cy - mz * sp * sy
    U[3][h] = mx * sp + mz * cp
    U[4][h] = P / (gamma - 1.0) + 0.5 * rho * vx * vx + A * sh * e["E"]
    if mhd:
        U[4][h] += 0.5 * (B[0] * B[0] + B[1] * B[1] + B[2] * B[2])
    return np.ascontiguousarray(U)


def sedov_box(n: int, ng: int, rng: np.random.Generator, gamma: float = 5.0 / 3.0, energy: float = 1.0,
              radius_cells: float = 3.0, dual_energy: bool = False) -> np.ndarray:
    """Sedov-like blast: energy deposited uniformly in cells within radius_cells of a random
    centre, ambient density 1 and pressure 1e-5, periodic box of side 1."""
    c = rng.uniform(0, n, size=3)
    idx = np.arange(n) + 0.5
    zz, yy, xx = np.meshgrid(idx, idx, idx, indexing="ij")
    r2 = (xx - c[0]) ** 2 + (yy - c[1]) ** 2 + (zz - c[2]) ** 2
    inside = r2 <= radius_cells ** 2
    dV = (1.0 / n) ** 3
    nin = max(int(inside.sum()), 1)
    eint = np.full((n, n, n), 1e-5 / (gamma - 1.0))
    eint[inside] = energy / (nin * dV)
    nf = n_fields(dual_energy)
    U = np.zeros((nf, n, n, n))
    U[0] = 1.0
    U[4] = eint
    if dual_energy:
        U[nf - 1] = eint
    return pad_periodic(U, ng)


def sod_box(n: int, ng: int, rng: np.random.Generator, gamma: float = 1.4, dual_energy: bool = False) -> np.ndarray:
    """3D Sod tube with the diaphragm normal in a random direction through the box centre."""
    nrm = rng.standard_normal(3)
    nrm /= np.linalg.norm(nrm)
    idx = (np.arange(n) + 0.5) / n - 0.5
    zz, yy, xx = np.meshgrid(idx, idx, idx, indexing="ij")
    s = nrm[0] * xx + nrm[1] * yy + nrm[2] * zz
    left = s < 0.0
    nf = n_fields(dual_energy)
    U = np.zeros((nf, n, n, n))
    U[0] = np.where(left, 1.0, 0.125)
    p = np.where(left, 1.0, 0.1)
    U[4] = p / (gamma - 1.0)
    if dual_energy:
        U[nf - 1] = U[4]
    return pad_periodic(U, ng)


def smooth_random_box(shape, ng: int, rng: np.random.Generator, gamma: float = 5.0 / 3.0,
                      dual_energy: bool = True, n_scalars: int = 0, amp: float = 0.3, mach: float = 0.8) -> np.ndarray:
    """Small smooth-but-structured periodic state for parity tests: a few random Fourier modes in
    density, velocity and pressure (non-cubic shapes allowed, shape = (nx, ny, nz) real cells)."""
    nx, ny, nz = shape
    x = (np.arange(nx) + 0.5) / nx
    y = (np.arange(ny) + 0.5) / ny
    z = (np.arange(nz) + 0.5) / nz
    zz, yy, xx = np.meshgrid(z, y, x, indexing="ij")

    def modes(k=3):
        f = np.zeros_like(xx)
        for _ in range(k):
            kx, ky, kz = rng.integers(1, 3, size=3)
            ph = rng.uniform(0, 2 * np.pi)
            f += rng.uniform(0.5, 1.0) * np.sin(2 * np.pi * (kx * xx + ky * yy + kz * zz) + ph)
        return f / k

    rho = 1.0 + amp * modes()
    p = 1.0 + amp * modes()
    cs = math.sqrt(gamma)
    v = np.stack([mach * cs * modes() for _ in range(3)])
    nf = n_fields(dual_energy, n_scalars=n_scalars)
    U = np.empty((nf, nz, ny, nx))
    U[0] = rho
    U[1:4] = rho * v
    U[4] = p / (gamma - 1.0) + 0.5 * rho * np.sum(v * v, axis=0)
    for s in range(n_scalars):
        U[5 + s] = rho * (1.0 + 0.5 * modes())
    if dual_energy:
        U[nf - 1] = p / (gamma - 1.0)
    return pad_periodic(U, ng)
