"""GPU parity: the fused CUDA step (through the C ABI) against the FP64 oracle.

The FP64 kernels keep the reference's operation order and are built with -fmad=false, so the
bar is bit-for-bit equality on real cells (tolerance 0 ULP).  Ghost cells are refilled by the
boundary kernel between steps and compared too where the test says so.
"""
import math

import numpy as np
import pytest

from helpers import real_slice

pytestmark = pytest.mark.gpu


def _gpu(cuda, arr):
    return cuda.from_numpy(np.ascontiguousarray(arr)).cuda()


def _scheme(recon="PPMC", solver="HLLC", de=True, ns=0, floor=True, gamma=5.0 / 3.0):
    from cholla_gb300 import integrator as I

    s = I.Scheme(reconstruction=recon, riemann_solver=solver, dual_energy=de, n_scalars=ns,
                 density_floor=floor, temperature_floor=False, gamma=gamma)
    I.set_scheme(s)
    return s


def _oracle_cfg(o, U, ng, recon, solver, de, ns, gamma, dx, floor=True):
    nf, nz, ny, nx = U.shape
    return o.config(nx, ny, nz, ng, nf, n_scalars=ns, de=de, recon={"PCM": o.PCM, "PLMC": o.PLMC, "PPMC": o.PPMC}[recon],
                    solver={"HLLC": o.HLLC, "ROE": o.ROE}[solver], density_floor_on=floor, gamma=gamma,
                    dx=dx[0], dy=dx[1], dz=dx[2])


def _assert_bitwise(got, want, ng, what=""):
    g = got[real_slice(ng)]
    w = want[real_slice(ng)]
    same = (g.view(np.int64) == w.view(np.int64)) | (np.isnan(g) & np.isnan(w))
    if not same.all():
        bad = np.argwhere(~same)
        i = tuple(bad[0])
        rel = np.max(np.abs(g - w) / np.maximum(np.abs(w), 1e-300))
        pytest.fail(f"{what}: {len(bad)} real-cell values differ; first at {i}: gpu {g[i]!r} oracle {w[i]!r}; "
                    f"max rel diff {rel:.3e}")


@pytest.mark.parametrize("recon", ["PCM", "PLMC", "PPMC"])
@pytest.mark.parametrize("solver", ["HLLC", "ROE"])
@pytest.mark.parametrize("de", [False, True])
def test_one_step_bitwise(cuda, oracle_lib, recon, solver, de):
    from cholla_gb300 import ics
    from cholla_gb300 import integrator as I

    o = oracle_lib
    ng = {"PCM": 2, "PLMC": 3, "PPMC": 4}[recon]
    rng = np.random.default_rng(7)
    U0 = ics.smooth_random_box((19, 13, 11), ng, rng, dual_energy=de)
    nf, nz, ny, nx = U0.shape
    dx = (1.0 / 19, 1.0 / 13, 1.0 / 11)
    dt = 0.2 * min(dx)
    _scheme(recon, solver, de)
    Ug = _gpu(cuda, U0)
    I.VL_Algorithm_3D_CUDA(Ug, None, nx, ny, nz, 0, 0, 0, ng, *dx, 0, 0, 0, dt, nf, 0, 0.0)
    cuda.cuda.synchronize()
    Uo = U0.copy()
    cfg = _oracle_cfg(o, Uo, ng, recon, solver, de, 0, 5.0 / 3.0, dx)
    o.vl_step_3d(cfg, Uo.reshape(-1), dt)
    _assert_bitwise(Ug.cpu().numpy(), Uo, ng, f"{recon}+{solver} de={de}")


@pytest.mark.parametrize("ns", [1, 2])
def test_scalars_bitwise(cuda, oracle_lib, ns):
    from cholla_gb300 import ics
    from cholla_gb300 import integrator as I

    o = oracle_lib
    ng = 4
    rng = np.random.default_rng(11)
    U0 = ics.smooth_random_box((12, 10, 9), ng, rng, dual_energy=True, n_scalars=ns)
    nf, nz, ny, nx = U0.shape
    dx = (1 / 12, 1 / 10, 1 / 9)
    dt = 0.2 * min(dx)
    _scheme("PPMC", "HLLC", True, ns)
    Ug = _gpu(cuda, U0)
    I.VL_Algorithm_3D_CUDA(Ug, None, nx, ny, nz, 0, 0, 0, ng, *dx, 0, 0, 0, dt, nf, 0, 0.0)
    Uo = U0.copy()
    o.vl_step_3d(_oracle_cfg(o, Uo, ng, "PPMC", "HLLC", True, ns, 5 / 3, dx), Uo.reshape(-1), dt)
    _assert_bitwise(Ug.cpu().numpy(), Uo, ng, f"scalars={ns}")


def test_multistep_turbulence_bitwise(cuda, oracle_lib):
    """Ten steps of the config-2 scheme (PPMC+HLLC+DE, floors) on a 24^3 turbulence box:
    boundary fill, step, temperature floor and CFL dt all on the GPU, compared bit for bit."""
    from cholla_gb300 import ics
    from cholla_gb300 import integrator as I

    o = oracle_lib
    n, ng, gamma = 24, 4, 5.0 / 3.0
    U0 = ics.turbulence_box(n, ng, gamma, seed=3)
    nf, N = U0.shape[0], U0.shape[1]
    dx = 1.0 / n
    s = I.Scheme(reconstruction="PPMC", riemann_solver="HLLC", dual_energy=True, density_floor=True,
                 temperature_floor=True, gamma=gamma)
    I.set_scheme(s)
    flags = (1, 1, 1, 1, 1, 1)
    Ug = _gpu(cuda, U0)
    Uo = U0.copy()
    cfg = _oracle_cfg(o, Uo, ng, "PPMC", "HLLC", True, 0, gamma, (dx, dx, dx))
    for step in range(10):
        dti_g = I.Calc_dt_GPU(Ug, N, N, N, ng, nf, dx, dx, dx, gamma)
        dti_o = o.calc_dt(cfg, Uo.reshape(-1))
        assert dti_g == dti_o, f"step {step}: dt reduction differs {dti_g!r} vs {dti_o!r}"
        dt = 0.3 / dti_g
        I.VL_Algorithm_3D_CUDA(Ug, None, N, N, N, 0, 0, 0, ng, dx, dx, dx, 0, 0, 0, dt, nf, 0, 0.0)
        I.Apply_Temperature_Floor(Ug, N, N, N, ng, nf, 0.0)
        I.Set_Boundaries(Ug, N, N, N, ng, nf, flags)
        o.vl_step_3d(cfg, Uo.reshape(-1), dt)
        o.temperature_floor(cfg, Uo.reshape(-1), 0.0)
        o.set_boundaries(cfg, Uo.reshape(-1), flags)
    got = Ug.cpu().numpy()
    same = got.view(np.int64) == Uo.view(np.int64)
    assert same.all(), f"{(~same).sum()} values differ after 10 steps (ghosts included)"


@pytest.mark.parametrize("flags", [(1, 1, 1, 1, 1, 1), (2, 2, 3, 3, 1, 1), (3, 3, 3, 3, 3, 3), (2, 3, 1, 1, 4, 2)])
def test_boundaries_bitwise(cuda, oracle_lib, flags):
    from cholla_gb300 import integrator as I

    o = oracle_lib
    rng = np.random.default_rng(5)
    ng, nf = 3, 6
    # every dimension keeps at least n_ghost real cells, so each ghost maps onto a real cell
    U0 = rng.uniform(0.1, 2.0, size=(nf, 10, 11, 12))
    U0[1:4] -= 1.0
    _scheme("PLMC", "HLLC", True)
    Ug = _gpu(cuda, U0)
    I.Set_Boundaries(Ug, 12, 11, 10, ng, nf, flags)
    Uo = U0.copy()
    o.set_boundaries(o.config(12, 11, 10, ng, nf, de=True), Uo.reshape(-1), flags)
    got = Ug.cpu().numpy()
    assert (got.view(np.int64) == Uo.view(np.int64)).all()


def test_sod_1d_bitwise_and_exact(cuda, oracle_lib):
    """Config 1: Sod tube, nx=100 + 4 ghosts, gamma=1.4, PPMC+HLLC, outflow boundaries,
    CFL 0.3 to t=0.2 -- GPU equals the oracle bit for bit at every step."""
    from cholla_gb300 import ics
    from cholla_gb300 import integrator as I

    o = oracle_lib
    ng, gamma = 4, 1.4
    U0, dx = ics.sod_1d(100, ng, gamma)
    nf, N = U0.shape
    I.set_scheme(I.Scheme(reconstruction="PPMC", riemann_solver="HLLC", dual_energy=False, density_floor=False,
                          temperature_floor=False, gamma=gamma))
    Ug = _gpu(cuda, U0)
    Uo = U0.copy()
    cfg = o.config(N, 1, 1, ng, nf, recon=o.PPMC, solver=o.HLLC, density_floor_on=False, gamma=gamma, dx=dx)
    flags = (3, 3, 0, 0, 0, 0)
    t = 0.0
    while t < 0.2:
        dti = I.Calc_dt_GPU(Ug, N, 1, 1, ng, nf, dx, dx, dx, gamma)
        assert dti == o.calc_dt(cfg, Uo.reshape(-1))
        dt = min(0.3 / dti, 0.2 - t)
        I.VL_Algorithm_1D_CUDA(Ug, N, 0, ng, dx, 0.0, dt, nf)
        I.Set_Boundaries(Ug, N, 1, 1, ng, nf, flags)
        o.vl_step_1d(cfg, Uo.reshape(-1), dt)
        o.set_boundaries(cfg, Uo.reshape(-1), flags)
        t += dt
    got = Ug.cpu().numpy()
    assert (got.view(np.int64) == Uo.view(np.int64)).all()
    from sod_exact import sod_exact

    x = (np.arange(100) + 0.5) * dx
    rho_ex = sod_exact(x, 0.2, gamma)[0]
    l1 = np.mean(np.abs(got[0, ng:-ng] - rho_ex))
    assert l1 < 0.01, f"L1 density error vs the exact solution {l1}"


def test_conservation_64(cuda):
    """Mass, momentum and energy of a periodic 64^3 turbulence box are conserved to roundoff
    over 5 steps (Mach 0.5 so no floor triggers; DE off so E is conserved by the flux form)."""
    from cholla_gb300 import ics
    from cholla_gb300 import integrator as I

    n, ng, gamma = 64, 4, 5.0 / 3.0
    U0 = ics.turbulence_box(n, ng, gamma, seed=9, mach=0.5, dual_energy=False)
    nf, N = U0.shape[0], U0.shape[1]
    dx = 1.0 / n
    I.set_scheme(I.Scheme(reconstruction="PPMC", riemann_solver="HLLC", dual_energy=False, density_floor=False,
                          temperature_floor=False, gamma=gamma))
    Ug = _gpu(cuda, U0)
    tot0 = Ug[:, ng:-ng, ng:-ng, ng:-ng].sum(dim=(1, 2, 3)).cpu().numpy()
    for _ in range(5):
        dt = 0.3 / I.Calc_dt_GPU(Ug, N, N, N, ng, nf, dx, dx, dx, gamma)
        I.VL_Algorithm_3D_CUDA(Ug, None, N, N, N, 0, 0, 0, ng, dx, dx, dx, 0, 0, 0, dt, nf, 0, 0.0)
        I.Set_Boundaries(Ug, N, N, N, ng, nf, (1, 1, 1, 1, 1, 1))
    tot = Ug[:, ng:-ng, ng:-ng, ng:-ng].sum(dim=(1, 2, 3)).cpu().numpy()
    scale = np.abs(U0[:, ng:-ng, ng:-ng, ng:-ng]).sum(axis=(1, 2, 3))
    drift = np.abs(tot - tot0) / scale
    assert np.all(drift[[0, 4]] < 1e-13), drift
    assert np.all(drift[1:4] < 1e-12), drift
