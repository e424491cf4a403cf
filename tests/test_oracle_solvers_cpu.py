"""The oracle's HLL and exact Riemann solvers (hll_cuda.cu, exact_cuda.cu), CPU only.  The GPU
kernels of these two make.type options are checked against these restatements in
tests/test_schemes_gpu.py and tests/test_fast_gpu.py; the restatements themselves are pinned here:

* HLL: the reference's HLLC known answer (a state against itself gives the pure pressure flux)
  under the reference's comparison rule; the upwind flux, bit for bit, when both wave speeds
  have one sign.
* exact: the flux of the sampled interface state against an independent Newton solution of
  the same Riemann problems (tests/sod_exact.py) for Toro's five test problems, to the
  reference's convergence tolerance (1e-6) and its single-precision fractional powers.
* both: a Sod tube run to t = 0.2 through the oracle's 1D step stays within 1% mean density
  error of the exact solution, and a periodic 3D box conserves mass to rounding.
* the weighted form in which the throughput kernels write the HLL flux: equal to the oracle's
  two-wave flux to FP64 rounding on random subsonic and supersonic faces.
"""
import json
import math
from pathlib import Path

import numpy as np
import pytest

from helpers import nearly_equal, real_slice

GOLD = json.loads((Path(__file__).parent / "golden" / "reference_fiducials.json").read_text())


def _interface(o, left, right, gamma, solver, de=False):
    """Flux of one interface between primitive states (d, vx, vy, vz, p); 1-cell arrays."""
    nf = 6 if de else 5
    QL, QR = np.zeros(nf), np.zeros(nf)
    for Q, (d, vx, vy, vz, p) in ((QL, left), (QR, right)):
        Q[:5] = [d, d * vx, d * vy, d * vz, p / (gamma - 1) + 0.5 * d * (vx * vx + vy * vy + vz * vz)]
        if de:
            Q[5] = p / (gamma - 1)
    cfg = o.config(1, 1, 1, 0, nf, de=de, recon=o.PCM, solver=solver, gamma=gamma)
    F = np.full(nf, -999.0)
    getattr(o.lib(), {o.HLL: "orc_hll", o.EXACT: "orc_exact"}[solver])(cfg, QL, QR, F, 0)
    return F


def test_hll_reference_known_answer(oracle_lib):
    o = oracle_lib
    for case in GOLD["hllc"]["cases"]:  # the same states give HLL the same flux
        F = _interface(o, case["left"], case["right"], case["gamma"], o.HLL)
        assert nearly_equal(np.array(case["fiducial"]), F).all(), F


@pytest.mark.parametrize("sign", [1.0, -1.0])
def test_hll_supersonic_is_upwind(oracle_lib, sign):
    """Both wave speeds of one sign: the flux is the upwind state's physical flux exactly."""
    o, g = oracle_lib, 1.4
    left, right = (1.0, sign * 5.0, 0.3, -0.2, 1.0), (0.5, sign * 4.0, -0.1, 0.4, 0.8)
    F = _interface(o, left, right, g, o.HLL)
    d, vx0, vy0, vz0, p0 = left if sign > 0 else right
    # the upwind side's physical flux from its conserved variables, in the solver's order
    mx, my, mz = d * vx0, d * vy0, d * vz0
    E = p0 / (g - 1) + 0.5 * d * (vx0 * vx0 + vy0 * vy0 + vz0 * vz0)
    vx, vy, vz = mx / d, my / d, mz / d
    p = max((E - 0.5 * d * (vx * vx + vy * vy + vz * vz)) * (g - 1.0), 1e-20)
    want = np.array([mx, mx * vx + p, my * vx, mz * vx, (E + p) * vx])
    assert np.array_equal(F, want), (F, want)


# Toro (2009), table 4.1: left and right (density, velocity, pressure), gamma = 1.4
TORO = [((1.0, 0.0, 1.0), (0.125, 0.0, 0.1)), ((1.0, -2.0, 0.4), (1.0, 2.0, 0.4)),
        ((1.0, 0.0, 1000.0), (1.0, 0.0, 0.01)), ((1.0, 0.0, 0.01), (1.0, 0.0, 100.0)),
        ((5.99924, 19.5975, 460.894), (5.99242, -6.19633, 46.0950))]


@pytest.mark.parametrize("k", range(len(TORO)), ids=[f"toro{k + 1}" for k in range(len(TORO))])
def test_exact_solver_matches_independent_solution(oracle_lib, k):
    from sod_exact import sod_exact

    o, g = oracle_lib, 1.4
    (dl, ul, pl), (dr, ur, pr) = TORO[k]
    F = _interface(o, (dl, ul, 0.0, 0.0, pl), (dr, ur, 0.0, 0.0, pr), g, o.EXACT)
    rho, u, p = (a[0] for a in sod_exact(np.array([0.5]), 1.0, g, (dl, ul, pl), (dr, ur, pr), 0.5))
    E = p / (g - 1) + 0.5 * rho * u * u
    want = np.array([rho * u, rho * u * u + p, 0.0, 0.0, (E + p) * u])
    scale = max(abs(pl), abs(pr), dl * ul * ul, dr * ur * ur, 1.0)
    assert np.allclose(F, want, rtol=1e-5, atol=1e-6 * scale), (F, want)


@pytest.mark.parametrize("solver", ["HLL", "EXACT"])
def test_sod_with_solver_matches_exact_solution(oracle_lib, solver):
    from cholla_gb300 import ics
    from sod_exact import sod_exact

    o = oracle_lib
    U1, dx = ics.sod_1d(100, 4, 1.4)
    nf, N = U1.shape
    if solver == "HLL":
        # the reference's 1D integrator has no HLL branch (VL_1D_cuda.cu:69-80): run the tube
        # through the 3D step, one real cell deep in y and z with periodic sides
        U = np.ascontiguousarray(np.broadcast_to(U1[:, None, None, :], (nf, 9, 9, N)))
        cfg = o.config(N, 9, 9, 4, nf, recon=o.PPMC, solver=o.HLL, density_floor_on=False, gamma=1.4, dx=dx, dy=dx,
                       dz=dx)
        step, flags = o.lib().orc_vl_step_3d, (3, 3, 1, 1, 1, 1)
    else:
        U = U1
        cfg = o.config(N, 1, 1, 4, nf, recon=o.PPMC, solver=o.EXACT, density_floor_on=False, gamma=1.4, dx=dx)
        step, flags = o.lib().orc_vl_step_1d, (3, 3, 0, 0, 0, 0)
    t = 0.0
    while t < 0.2:
        dt = min(0.3 / o.calc_dt(cfg, U.reshape(-1)), 0.2 - t)
        assert step(cfg, U.reshape(-1), dt) == 0
        o.set_boundaries(cfg, U.reshape(-1), flags)
        t += dt
    x = (np.arange(100) + 0.5) * dx
    rho = sod_exact(x, 0.2, 1.4)[0]
    assert np.mean(np.abs(U.reshape(nf, -1, N)[0, 0, 4:-4] - rho)) < 0.01


@pytest.mark.parametrize("solver", ["HLL", "EXACT"])
def test_solver_conserves_on_periodic_box(oracle_lib, solver):
    from cholla_gb300 import ics

    o = oracle_lib
    U = ics.smooth_random_box((12, 10, 8), 4, np.random.default_rng(3), dual_energy=True)
    nf, nz, ny, nx = U.shape
    cfg = o.config(nx, ny, nz, 4, nf, de=True, recon=o.PPMC, solver=getattr(o, solver), gamma=5 / 3, dx=1 / 12,
                   dy=1 / 10, dz=1 / 8)
    tot0 = U[real_slice(4)][:5].sum(axis=(1, 2, 3))
    for _ in range(3):
        dt = 0.3 / o.calc_dt(cfg, U.reshape(-1))
        assert o.lib().orc_vl_step_3d(cfg, U.reshape(-1), dt) == 0
        o.set_boundaries(cfg, U.reshape(-1), (1,) * 6)
    tot = U[real_slice(4)][:5].sum(axis=(1, 2, 3))
    assert np.all(np.isfinite(U))
    assert np.allclose(tot, tot0, rtol=1e-12, atol=1e-12 * math.fsum(np.abs(tot0)))


def _hll_weighted(left, right, g):
    """The fast forms' HLL (hf::hll_q in cholla_gb300/csrc/hydro_fast.cuh) restated in numpy: the
    two-wave flux as dL bL XL + dR bR XR plus the pressure terms, with selected weights on
    supersonic faces."""
    (dl, vl, t1l, t2l, pl), (dr, vr, t1r, t2r, pr) = left, right
    El = pl / (g - 1) + 0.5 * dl * (vl * vl + t1l * t1l + t2l * t2l)
    Er = pr / (g - 1) + 0.5 * dr * (vr * vr + t1r * t1r + t2r * t2r)
    cl, cr = math.sqrt(g * pl / dl), math.sqrt(g * pr / dr)
    Sl, Sr = min(vr - cr, vl - cl), max(vl + cl, vr + cr)
    dSl, dSr = Sl - vl, Sr - vr
    inv = 1.0 / max(Sr - Sl, 1e-30)
    if Sl > 0:
        wl, wr, bl, br = 1.0, 0.0, vl, 0.0
    elif Sr < 0:
        wl, wr, bl, br = 0.0, 1.0, 0.0, vr
    else:
        wl, wr, bl, br = Sr * inv, -Sl * inv, -(Sr * dSl) * inv, (Sl * dSr) * inv
    al, ar = dl * bl, dr * br
    return np.array([al + ar, al * vl + ar * vr + (wl * pl + wr * pr), al * t1l + ar * t1r, al * t2l + ar * t2r,
                     bl * El + br * Er + (wl * pl * vl + wr * pr * vr)])


def test_weighted_hll_form_equals_the_two_wave_flux(oracle_lib):
    """The algebra of the fast forms' HLL: on random states (subsonic and supersonic, either
    direction) the weighted form equals the oracle's (Sr FL - Sl FR + Sl Sr (UR - UL)) / (Sr - Sl)
    to FP64 rounding (relative to the flux's scale)."""
    o, g = oracle_lib, 1.4
    rng = np.random.default_rng(5)
    worst = 0.0
    for _ in range(400):
        left = (rng.uniform(0.1, 2), rng.normal(0, 3), rng.normal(0, 1), rng.normal(0, 1), rng.uniform(0.1, 2))
        right = (rng.uniform(0.1, 2), rng.normal(0, 3), rng.normal(0, 1), rng.normal(0, 1), rng.uniform(0.1, 2))
        want = _interface(o, left, right, g, o.HLL)
        got = _hll_weighted(left, right, g)
        scale = max(np.abs(want).max(), 1.0)
        worst = max(worst, float(np.abs(got - want).max() / scale))
    assert worst < 1e-13, worst
