"""Shared helpers for the test suite (comparison rules of the reference's unit tests)."""
from __future__ import annotations

import math

import numpy as np


def ulp_diff(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    ia = np.asarray(a, dtype=np.float64).view(np.int64)
    ib = np.asarray(b, dtype=np.float64).view(np.int64)
    # map sign-magnitude to two's-complement ordering
    ia = np.where(ia < 0, np.int64(-0x8000000000000000) - ia, ia)
    ib = np.where(ib < 0, np.int64(-0x8000000000000000) - ib, ib)
    return np.abs(ia - ib)


def nearly_equal(fid, test, abs_eps: float = 1e-14, ulps: int = 4) -> np.ndarray:
    """testing_utilities::nearlyEqualDbl (src/utils/testing_utilities.h:85-86): equal when the
    absolute difference is <= 1e-14 or the two doubles are within 4 ULP."""
    fid = np.asarray(fid, dtype=np.float64)
    test = np.asarray(test, dtype=np.float64)
    return (np.abs(fid - test) <= abs_eps) | (ulp_diff(fid, test) <= ulps)


def real_slice(ng: int, one_d: bool = False):
    if one_d:
        return (slice(None), slice(ng, -ng))
    return (slice(None), slice(ng, -ng), slice(ng, -ng), slice(ng, -ng))


# ---- the reference's linear-wave system tests (src/system_tests/hydro_system_tests.cpp) ----
C_CFL = 0.3  # src/grid/grid3D.cpp:157


def linear_wave_setup(setup: dict, wave: dict, ng: int):
    """(U, (Nx, Ny, Nz), dx, tout) of one linear-wave system test: 2N x N x N real cells on a
    [0, 2 domain] x [0, domain]^2 box, rho = 1, P = 1 / gamma, amplitude 1e-6, run for the time
    the wave needs to cross the box (2 domain / wave speed)."""
    from cholla_gb300 import ics

    N, domain, gamma = int(setup["N"]), setup["domain"], setup["gamma"]
    dx = 2 * domain / (2 * N)
    U = ics.linear_wave(2 * N, N, N, ng, dx, dx, dx, gamma=gamma, rho=1.0, P=1.0 / gamma, A=1e-6, eigen=wave["eigen"],
                        vx=wave["vx"])
    return U, (2 * N + 2 * ng, N + 2 * ng, N + 2 * ng), dx, 2 * domain / wave["wave_speed"]


def run_reference_loop(step, calc_dti, fill_ghosts, tout: float):
    """The reference's main loop (src/main.cpp:247-300): dt = C_cfl / max inverse crossing time,
    clamped so the last step lands on tout, then the step, t += dt, the ghost fill.  Returns
    (number of steps, final time)."""
    dti, t, n = calc_dti(), 0.0, 0
    while t < tout:
        dt = C_CFL / dti
        if t + dt > tout:
            dt = tout - t
        step(dt)
        dti = calc_dti()
        t += dt
        n += 1
        fill_ghosts()
    return n, t


def l1_errors(U0: np.ndarray, U1: np.ndarray, ng: int, n_hydro: int = 5):
    """Per-field mean absolute change over the real cells (the system tests' L1 error, GasEnergy
    excluded), the norm of that vector and the largest single change."""
    rs = real_slice(ng)
    d = np.abs(U1[rs][:n_hydro] - U0[rs][:n_hydro])
    l1 = np.array([math.fsum(f.ravel()) / f.size for f in d])
    return l1, float(np.sqrt((l1 ** 2).sum())), float(d.max())


def mhd_wave_setup(sysd: dict, case: dict, angle, N: int | None = None):
    """(real cells per side, dx, tout, pitch, yaw) of one MHD linear-wave system test
    (src/system_tests/mhd_system_tests.cpp:39-121): N^3 real cells of side 0.5 with the wave's
    direction (1 x, 2 y, 3 z) doubled, run for the time the wave needs to cross the long side."""
    pitch, yaw, domain, direction = angle
    N = N or case["N"]
    n = [N, N, N]
    n[int(direction) - 1] *= 2
    return n, domain / N, 2 * domain / case["wave_speed"], pitch, yaw


def mhd_wave_state(sysd: dict, case: dict, angle, ng: int, N: int | None = None):
    """(U, padded shape, dx, tout): the Linear_Wave state of the test, background B = (1, 1.5, 0)
    rotated with the wave by (pitch, yaw)."""
    from cholla_gb300 import ics

    n, dx, tout, pitch, yaw = mhd_wave_setup(sysd, case, angle, N)
    U = ics.linear_wave(n[0], n[1], n[2], ng, dx, dx, dx, gamma=sysd["gamma"], rho=1.0, P=1.0 / sysd["gamma"],
                        A=sysd["amplitude"], eigen=case["eigen"], vx=case["vx"], B=tuple(sysd["B"]), pitch=pitch,
                        yaw=yaw, mhd=True)
    return U, (n[0] + 2 * ng, n[1] + 2 * ng, n[2] + 2 * ng), dx, tout


def l1_errors_mhd(U0: np.ndarray, U1: np.ndarray, ng: int):
    """The system tests' L1 errors for an MHD state: the five hydro fields over the real cells,
    each face field over the faces the reference writes out (one more, the lower face of the
    first real cell, along its own direction); the norm of the eight and the largest change."""
    l1h, _, worst = l1_errors(U0, U1, ng)
    out = list(l1h)
    for k in range(3):
        sl = [slice(ng, -ng)] * 3  # [z, y, x]
        sl[2 - k] = slice(ng - 1, -ng)
        d = np.abs(U1[(5 + k, *sl)] - U0[(5 + k, *sl)])
        out.append(math.fsum(d.ravel()) / d.size)
        worst = max(worst, float(d.max()))
    l1 = np.array(out)
    return l1, float(np.sqrt((l1 ** 2).sum())), worst


def constant_state(st: dict, ng: int, mhd: bool = False, dual_energy: bool = False):
    """(U, padded shape, dx) of the Constant initial condition (src/grid/initial_conditions.cpp:
    180-238) on the settings of a system-test input file: uniform rho, momenta rho v, energy
    P / (gamma - 1) + rho v^2 / 2 (without a magnetic term, as the reference writes it) and
    uniform face fields; filled everywhere, which the periodic ghost fill would give anyway."""
    n = [int(st["nx"]), int(st["ny"]), int(st["nz"])]
    shape = tuple(k + 2 * ng for k in n)
    nf = 5 + (3 if mhd else 0) + (1 if dual_energy else 0)
    U = np.zeros((nf, shape[2], shape[1], shape[0]))
    rho, g = st["rho"], st["gamma"]
    v = (st["vx"], st["vy"], st["vz"])
    U[0] = rho
    for k in range(3):
        U[1 + k] = rho * v[k]
    U[4] = st["P"] / (g - 1.0) + 0.5 * rho * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2])
    if mhd:
        U[5], U[6], U[7] = st["Bx"], st["By"], st["Bz"]
    if dual_energy:
        U[nf - 1] = st["P"] / (g - 1.0)
    return np.ascontiguousarray(U), shape, st["xlen"] / n[0]
