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
