"""The FP64 oracle against the reference itself, run on the CPU (CPU only).

oracle/build_ref_host.sh compiles the reference's VL integrators and kernels, unchanged from its
source tree, as host C++ (one library per make.type scheme: reconstruction, Riemann solver, dual
energy, scalar, MHD).  These tests run a step of each scheme through both and require the real
cells to be equal bit for bit:

* 3D steps (VL_3D_cuda.cu:38) on a seeded 16^3 turbulence box (hydro) or a seeded MHD box, two
  steps with a periodic ghost fill between them;
* 2D steps (VL_2D_cuda.cu:25) on a 24 x 24 periodic slab of the same box, two steps;
* 1D steps (VL_1D_cuda.cu:30) on the Sod tube, ten steps with outflow ghosts;
* single launches of the primitive-limited reconstructions PLMP_cuda and PPMP_cuda along each
  direction (every interface value they write);
* single launches of the HLLC, Roe, HLL and exact flux kernels on random interface states;
* the ghost fill (SetGhostCells per face) for periodic, reflective, outflow and mixed faces;
* the temperature floor (Apply_Temperature_Floor) with and without dual energy;
* a full linear-sound-wave crossing in the PPMP build (214 steps), the case where the reference
  misses its own largest-error bound.

The MHD schemes' characteristic projection uses 1/sqrt and 1/hypot on both sides (CUDA's rsqrt
and rhypot have no host counterpart), so those two compare the same arithmetic.
"""
import json
from pathlib import Path

import numpy as np
import pytest

from helpers import linear_wave_setup, run_reference_loop

HYDRO = ["ppmc_hllc_de", "ppmc_hllc", "ppmc_hllc_de_scalar", "plmc_hllc", "pcm_hllc_de", "ppmc_roe_de", "ppmc_hll_de",
         "plmp_hllc", "plmp_hllc_de", "plmp_hll", "ppmp_hllc_de", "ppmp_hllc", "ppmp_roe"]
MHD = ["mhd_plmc_hlld", "mhd_ppmc_hlld"]
GAMMA = 5.0 / 3.0


def _scheme(o, name):
    parts = name.split("_")
    mhd = parts[0] == "mhd"
    if mhd:
        parts = parts[1:]
    return dict(mhd=mhd, recon=getattr(o, parts[0].upper()), solver=getattr(o, parts[1].upper()), de="de" in parts,
                n_scalars=int("scalar" in parts))


def _same(a, b):
    return bool(np.all((a.view(np.int64) == b.view(np.int64)) | (np.isnan(a) & np.isnan(b))))


def _real(U, ng, dims):
    return U[(slice(None),) + (slice(ng, -ng),) * dims]


def _hydro_box(n, ng, de, n_scalars):
    from cholla_gb300 import ics

    U = ics.turbulence_box(n, ng, GAMMA, seed=5, dual_energy=de)
    if n_scalars:  # a passive scalar density between the energy and GasEnergy fields
        U = np.concatenate([U[:5], (0.3 * U[0] * (1.0 + 0.5 * np.sin(7 * U[1])))[None], U[5:]])
    return np.ascontiguousarray(U)


@pytest.mark.parametrize("name", HYDRO + MHD)
def test_step_3d_matches_reference(oracle_lib, ref_host, name):
    from cholla_gb300 import ics

    o, s = oracle_lib, _scheme(oracle_lib, name)
    n, ng = 16, 4
    U = ics.mhd_box(n, ng, GAMMA, seed=2) if s["mhd"] else _hydro_box(n, ng, s["de"], s["n_scalars"])
    nf, N = U.shape[0], U.shape[1]
    dx = 1.0 / n
    cfg = o.config(N, N, N, ng, nf, gamma=GAMMA, dx=dx, dy=dx, dz=dx, **s)
    Uo, Ur = U.reshape(nf, -1).copy(), U.reshape(nf, -1).copy()
    for _ in range(2):
        dt = 0.3 / o.calc_dt(cfg, Uo)
        o.vl_step_3d(cfg, Uo, dt)
        ref_host.vl_step_3d(name, Ur, N, N, N, ng, dx, dx, dx, dt, GAMMA)
        o.set_boundaries(cfg, Uo, (1,) * 6)
        o.set_boundaries(cfg, Ur, (1,) * 6)
    a, b = _real(Uo.reshape(nf, N, N, N), ng, 3), _real(Ur.reshape(nf, N, N, N), ng, 3)
    assert np.all(np.isfinite(a)) and not np.array_equal(a, _real(U, ng, 3))
    assert _same(a, b), np.abs(a - b).max(axis=(1, 2, 3))


def _wrap_2d(U, ng):
    real = U[:, ng:-ng, ng:-ng]
    return np.ascontiguousarray(np.pad(real, ((0, 0), (ng, ng), (ng, ng)), mode="wrap"))


@pytest.mark.parametrize("name", [h for h in HYDRO if "hll_" not in h + "_"])
def test_step_2d_matches_reference(oracle_lib, ref_host, name):
    """The 2D integrator has no HLL branch (VL_2D_cuda.cu:49-66), so the HLL schemes are absent."""
    o, s = oracle_lib, _scheme(oracle_lib, name)
    n, ng = 24, 4
    U3 = _hydro_box(n, ng, s["de"], s["n_scalars"])
    nf, N = U3.shape[0], U3.shape[1]
    U = _wrap_2d(U3[:, N // 2], ng)  # one z plane, periodic in x and y
    dx = 1.0 / n
    cfg = o.config(N, N, 1, ng, nf, gamma=GAMMA, dx=dx, dy=dx, dz=dx, **s)
    Uo, Ur = U.reshape(nf, -1).copy(), U.reshape(nf, -1).copy()
    for _ in range(2):
        dt = 0.3 / o.calc_dt(cfg, Uo)
        o.vl_step_2d(cfg, Uo, dt)
        ref_host.vl_step_2d(name, Ur, N, N, ng, dx, dx, dt, GAMMA)
        Uo[:] = _wrap_2d(Uo.reshape(nf, N, N), ng).reshape(nf, -1)
        Ur[:] = _wrap_2d(Ur.reshape(nf, N, N), ng).reshape(nf, -1)
    a, b = _real(Uo.reshape(nf, N, N), ng, 2), _real(Ur.reshape(nf, N, N), ng, 2)
    assert np.all(np.isfinite(a)) and not np.array_equal(a, _real(U, ng, 2))
    assert _same(a, b), np.abs(a - b).max(axis=(1, 2))


@pytest.mark.parametrize("name", [h for h in HYDRO if "hll_" not in h + "_"])
def test_step_1d_matches_reference(oracle_lib, ref_host, name):
    """Sod tube, outflow ghosts.  The 1D integrator has no HLL branch (VL_1D_cuda.cu:69-80)."""
    from cholla_gb300 import ics

    o, s = oracle_lib, _scheme(oracle_lib, name)
    ng = 4
    U, dx = ics.sod_1d(100, ng, GAMMA, dual_energy=s["de"])
    if s["n_scalars"]:
        U = np.concatenate([U[:5], (0.3 * U[0])[None], U[5:]])
    nf, N = U.shape
    cfg = o.config(N, 1, 1, ng, nf, gamma=GAMMA, dx=dx, **s)
    Uo, Ur = np.ascontiguousarray(U).copy(), np.ascontiguousarray(U).copy()
    for _ in range(10):
        dt = 0.3 / o.calc_dt(cfg, Uo)
        o.vl_step_1d(cfg, Uo.reshape(-1), dt)
        ref_host.vl_step_1d(name, Ur.reshape(-1), N, ng, dx, dt, GAMMA)
        o.set_boundaries(cfg, Uo.reshape(-1), (3, 3, 0, 0, 0, 0))
        o.set_boundaries(cfg, Ur.reshape(-1), (3, 3, 0, 0, 0, 0))
    assert _same(Uo[:, ng:-ng], Ur[:, ng:-ng]), np.abs(Uo - Ur)[:, ng:-ng].max(axis=1)


@pytest.mark.parametrize("kind", ["plmp", "ppmp"])
@pytest.mark.parametrize("de", [False, True])
def test_primitive_reconstruction_matches_reference(oracle_lib, ref_host, kind, de):
    o = oracle_lib
    name = f"{kind}_hllc" + ("_de" if de else "")
    U = _hydro_box(12, 4, de, 0)
    nf, N = U.shape[0], U.shape[1]
    cfg = o.config(N, N, N, 4, nf, de=de, recon=getattr(o, kind.upper()), gamma=GAMMA)
    flat = U.reshape(nf, -1)
    for direction in range(3):
        QLo, QRo, QLr, QRr = (np.zeros_like(flat) for _ in range(4))
        getattr(o.lib(), f"orc_{kind}")(cfg, flat, QLo, QRo, direction)
        ref_host.reconstruct(name, kind, flat, QLr, QRr, N, N, N, 4, 1.0 / 12, 0.01, GAMMA, direction)
        assert np.count_nonzero(QLr) > 0.6 * QLr.size
        assert _same(QLo, QLr) and _same(QRo, QRr), direction


def test_ppmp_sound_wave_crossing_matches_reference(oracle_lib, ref_host):
    """The reference's linear sound wave (hydro_system_tests.cpp:160-306) in the PPMP build, over
    the whole 214-step crossing: the oracle ends on the reference's state bit for bit."""
    o = oracle_lib
    sysd = json.loads((Path(__file__).parent / "golden" / "reference_fiducials.json").read_text())["hydro_system"]
    lw = sysd["linear_waves"]["PPMP"]
    w = lw["waves"]["SoundWaveRightMovingCorrectInputExpectCorrectOutput"]
    ng, gamma = 4, lw["setup"]["gamma"]
    U, (Nx, Ny, Nz), dx, tout = linear_wave_setup(lw["setup"], w, ng)
    cfg = o.config(Nx, Ny, Nz, ng, 5, recon=o.PPMP, solver=o.HLLC, gamma=gamma, dx=dx, dy=dx, dz=dx)
    Ur = np.ascontiguousarray(U.ravel())
    o.set_boundaries(cfg, Ur, (1,) * 6)
    Uo = Ur.copy()
    steps = []
    for U_, step in ((Uo, lambda dt: o.vl_step_3d(cfg, Uo, dt)),
                     (Ur, lambda dt: ref_host.vl_step_3d("ppmp_hllc", Ur, Nx, Ny, Nz, ng, dx, dx, dx, dt, gamma))):
        steps.append(run_reference_loop(step, lambda U_=U_: o.calc_dt(cfg, U_),
                                        lambda U_=U_: o.set_boundaries(cfg, U_, (1,) * 6), tout))
    assert steps[0] == steps[1] == (w["n_steps"], tout)
    assert _same(Uo, Ur)


@pytest.mark.parametrize("de", [False, True])
@pytest.mark.parametrize("solver", ["HLLC", "ROE", "HLL", "EXACT"])
def test_riemann_kernel_matches_reference(oracle_lib, ref_host, solver, de):
    """One launch of each hydro flux kernel on seeded random interface states (density 0.1-10,
    velocities within +-1, pressure 1-10: strong jumps, but no state pair that opens a vacuum,
    where the reference's exact solver prints a message), every direction.  The exact solver's kernel is
    built on its own (its integrators do not compile); both sides evaluate its single-precision
    powf on the host, so they agree bit for bit but only approximate the GPU's powf."""
    o = oracle_lib
    scheme = "pcm_exact_de" if de else "pcm_exact"
    n, ng = 10, 2
    nf = 6 if de else 5
    size = n ** 3
    rng = np.random.default_rng(11)

    def states():
        d = rng.uniform(0.1, 10.0, size)
        v = rng.uniform(-1.0, 1.0, (3, size))
        p = rng.uniform(1.0, 10.0, size)
        E = p / (GAMMA - 1.0) + 0.5 * d * (v ** 2).sum(axis=0)
        fields = [d, d * v[0], d * v[1], d * v[2], E] + ([p / (GAMMA - 1.0)] if de else [])
        return np.ascontiguousarray(np.stack(fields))

    QL, QR = states(), states()
    cfg = o.config(n, n, n, ng, nf, de=de, solver=getattr(o, solver), gamma=GAMMA)
    for direction in range(3):
        Fo, Fr = np.zeros_like(QL), np.zeros_like(QL)
        getattr(o.lib(), f"orc_{solver.lower()}")(cfg, QL, QR, Fo, direction)
        ref_host.riemann(scheme, getattr(o, solver), QL, QR, Fr, n, n, n, ng, GAMMA, direction)
        assert np.count_nonzero(Fr) > 0.5 * Fr.size
        assert _same(Fo, Fr), (direction, np.abs(Fo - Fr).max(axis=1))


@pytest.mark.parametrize("flags", [(1,) * 6, (2,) * 6, (3,) * 6, (3, 2, 1, 1, 2, 3)])
@pytest.mark.parametrize("name", ["ppmc_hllc_de", "mhd_plmc_hlld"])
def test_ghost_fill_matches_reference(oracle_lib, ref_host, name, flags):
    """The ghost fill between steps (SetGhostCellsKernel, grid/cuda_boundaries.cu:71-149):
    periodic (1), reflective (2) and outflow (3, with the hydro build's diode on the normal
    momentum) faces on a random box whose ghost cells start random; every cell compared, ghosts
    included.  The MHD build copies without the diode."""
    o = oracle_lib
    mhd = name.startswith("mhd")
    rng = np.random.default_rng(sum(flags) + 7 * mhd)
    nx, ny, nz, ng = 10 + 8, 9 + 8, 8 + 8, 4
    nf = 8 if mhd else 6
    U = rng.uniform(-1.0, 1.0, (nf, nz, ny, nx))
    U[0] = rng.uniform(0.5, 2.0, (nz, ny, nx))
    U[4] = rng.uniform(5.0, 9.0, (nz, ny, nx))
    cfg = o.config(nx, ny, nz, ng, nf, de=not mhd, mhd=mhd, recon=o.PLMC if mhd else o.PPMC,
                   solver=o.HLLD if mhd else o.HLLC, gamma=GAMMA)
    Uo, Ur = U.reshape(nf, -1).copy(), U.reshape(nf, -1).copy()
    o.set_boundaries(cfg, Uo, flags)
    ref_host.set_boundaries(name, Ur, nx, ny, nz, ng, flags)
    assert not np.array_equal(Uo, U.reshape(nf, -1))
    assert _same(Uo, Ur), np.abs(Uo - Ur).max(axis=1)


def test_ghost_fill_1d_matches_reference(oracle_lib, ref_host):
    from cholla_gb300 import ics

    o = oracle_lib
    U, dx = ics.sod_1d(100, 4, GAMMA)
    U[1] = np.linspace(-1.0, 1.0, U.shape[1])  # inflow at both ends: the diode acts
    nf, N = U.shape
    cfg = o.config(N, 1, 1, 4, nf, gamma=GAMMA, dx=dx)
    Uo, Ur = np.ascontiguousarray(U), np.ascontiguousarray(U).copy()
    o.set_boundaries(cfg, Uo.reshape(-1), (3, 3, 0, 0, 0, 0))
    ref_host.set_boundaries("ppmc_hllc", Ur.reshape(-1), N, 1, 1, 4, (3, 3, 0, 0, 0, 0))
    assert _same(Uo, Ur)


@pytest.mark.parametrize("name", ["ppmc_hllc", "ppmc_hllc_de"])
def test_temperature_floor_matches_reference(oracle_lib, ref_host, name):
    """Apply_Temperature_Floor (hydro_cuda.cu:1103-1153) with a floor that about half the cells
    are under: both the total energy and, with dual energy, GasEnergy are raised there."""
    o = oracle_lib
    de = name.endswith("_de")
    U = _hydro_box(12, 4, de, 0)
    nf, N = U.shape[0], U.shape[1]
    cfg = o.config(N, N, N, 4, nf, de=de, gamma=GAMMA)
    Uo, Ur = U.reshape(nf, -1).copy(), U.reshape(nf, -1).copy()
    eint = (U[4] - 0.5 * (U[1] ** 2 + U[2] ** 2 + U[3] ** 2) / U[0]).ravel()
    floor = float(np.median(eint))
    o.temperature_floor(cfg, Uo, floor)
    ref_host.temperature_floor(name, Ur, N, N, N, 4, floor)
    assert not np.array_equal(Uo, U.reshape(nf, -1))
    assert _same(Uo, Ur)
