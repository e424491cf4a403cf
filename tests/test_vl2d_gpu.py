"""The 2D VL step (cgb_vl_algorithm_2d, replacing VL_Algorithm_2D_CUDA of
src/integrators/VL_2D_cuda.cu) on the GPU against the FP64 oracle's orc_vl_step_2d, which equals
the host-run reference's 2D integrator bit for bit.

Every reconstruction the 2D integrator supports (with PCM its corrector reuses the predictor's
fluxes), with HLLC, Roe and the exact solver (the 2D integrator has no HLL branch), with and
without dual energy: bit for bit on real cells, except with the exact solver, whose powf is CUDA's
here and glibc's in the oracle (relative L1 <= 1e-7).  Multi-step runs include the 2D CFL reduction
(Calc_dt_2D), the periodic ghost fill and the box engine.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NG = {"PCM": 2, "PLMC": 3, "PPMC": 4, "PLMP": 3, "PPMP": 4}


def _state(nx, ny, ng, de, seed, ns=0, gamma=5 / 3):
    """A smooth random 2D state: Fourier modes in density, velocities and pressure, one cell deep."""
    from cholla_gb300 import ics

    rng = np.random.default_rng(seed)
    U3 = ics.smooth_random_box((nx, ny, 1), ng, rng, dual_energy=de, n_scalars=ns, gamma=gamma)
    # keep the middle z layer of the padded 3D box: a 2D box of (nx + 2 ng) x (ny + 2 ng) x 1
    return np.ascontiguousarray(U3[:, ng:ng + 1, :, :])


def _real(U, ng):
    return U[:, :, ng:-ng, ng:-ng]


def _cfg(o, U, ng, recon, solver, de, dx, dy, ns=0, gamma=5 / 3):
    nf, nz, ny, nx = U.shape
    return o.config(nx, ny, 1, ng, nf, n_scalars=ns, de=de, recon=getattr(o, recon), solver=getattr(o, solver),
                    gamma=gamma, dx=dx, dy=dy, dz=dx)


def _check(got, want, ng, solver, what):
    g, w = _real(got, ng), _real(want, ng)
    if solver == "EXACT":
        err = np.abs(g - w).sum(axis=(1, 2, 3)) / np.abs(w).sum(axis=(1, 2, 3))
        assert np.all(err <= 1e-7), f"{what}: relative L1 {err}"
    else:
        same = g.view(np.int64) == w.view(np.int64)
        assert same.all(), f"{what}: {(~same).sum()} real values differ, max |diff| {np.abs(g - w).max():.3e}"


@pytest.mark.parametrize("recon", ["PCM", "PLMC", "PPMC", "PLMP", "PPMP"])
@pytest.mark.parametrize("solver", ["HLLC", "ROE", "EXACT"])
@pytest.mark.parametrize("de", [False, True])
def test_2d_one_step(cuda, oracle_lib, recon, solver, de):
    from cholla_gb300 import integrator as I

    o = oracle_lib
    ng = NG[recon]
    U0 = _state(37, 29, ng, de, seed=51)
    nf, _, ny, nx = U0.shape
    dx, dy = 1 / 37, 1 / 29
    dt = 0.2 * min(dx, dy)
    I.set_scheme(I.Scheme(reconstruction=recon, riemann_solver=solver, dual_energy=de, temperature_floor=False))
    try:
        Ug = cuda.from_numpy(U0.copy()).cuda()
        I.VL_Algorithm_2D_CUDA(Ug, nx, ny, 0, 0, ng, dx, dy, 0.0, 0.0, dt, nf)
        cuda.cuda.synchronize()
        Uo = U0.copy()
        assert o.vl_step_2d(_cfg(o, Uo, ng, recon, solver, de, dx, dy), Uo.reshape(-1), dt) is None
        _check(Ug.cpu().numpy(), Uo, ng, solver, f"{recon}+{solver} de={de}")
    finally:
        I.set_scheme(I.Scheme())


@pytest.mark.parametrize("recon,solver,ns", [("PPMC", "HLLC", 0), ("PLMP", "ROE", 2), ("PCM", "HLLC", 1)])
def test_2d_multistep_with_dt_and_ghosts(cuda, oracle_lib, recon, solver, ns):
    from cholla_gb300 import integrator as I

    o = oracle_lib
    ng, gamma = NG[recon], 5 / 3
    U0 = _state(40, 24, ng, True, seed=52, ns=ns)
    nf, _, ny, nx = U0.shape
    dx, dy = 1 / 40, 1 / 24
    I.set_scheme(I.Scheme(reconstruction=recon, riemann_solver=solver, dual_energy=True, n_scalars=ns))
    try:
        Ug = cuda.from_numpy(U0.copy()).cuda()
        Uo = U0.copy()
        cfg = _cfg(o, Uo, ng, recon, solver, True, dx, dy, ns=ns)
        flags = (1, 1, 1, 1, 0, 0)
        for step in range(8):
            dti = I.Calc_dt_GPU(Ug, nx, ny, 1, ng, nf, dx, dy, dx, gamma)
            assert dti == o.calc_dt(cfg, Uo.reshape(-1)), f"step {step}: 2D dt reduction differs"
            dt = 0.3 / dti
            I.VL_Algorithm_2D_CUDA(Ug, nx, ny, 0, 0, ng, dx, dy, 0.0, 0.0, dt, nf)
            I.Set_Boundaries(Ug, nx, ny, 1, ng, nf, flags)
            o.vl_step_2d(cfg, Uo.reshape(-1), dt)
            o.set_boundaries(cfg, Uo.reshape(-1), flags)
        cuda.cuda.synchronize()
        _check(Ug.cpu().numpy(), Uo, ng, solver, f"{recon}+{solver} 8 steps")
    finally:
        I.set_scheme(I.Scheme())


def test_2d_box_engine_equals_dropin(cuda):
    from cholla_gb300 import integrator as I
    from cholla_gb300.engine import Box

    ng, gamma = 4, 5 / 3
    U0 = _state(32, 32, ng, True, seed=53)
    nf, _, ny, nx = U0.shape
    dx = 1 / 32
    s = I.Scheme(reconstruction="PPMC", riemann_solver="HLLC", dual_energy=True)
    box = Box(nx, ny, 1, ng, dx, dx, dx, s, flags=(1, 1, 1, 1, 0, 0))
    Ub = cuda.from_numpy(U0.copy()).cuda()
    box.advance(Ub, 5, 0.3)
    t_box, _ = box.time()
    box.close()
    I.set_scheme(s)
    try:
        Ud = cuda.from_numpy(U0.copy()).cuda()
        t = 0.0
        for _ in range(5):
            I.Set_Boundaries(Ud, nx, ny, 1, ng, nf, (1, 1, 1, 1, 0, 0))
            dt = 0.3 / I.Calc_dt_GPU(Ud, nx, ny, 1, ng, nf, dx, dx, dx, gamma)
            I.VL_Algorithm_2D_CUDA(Ud, nx, ny, 0, 0, ng, dx, dx, 0.0, 0.0, dt, nf)
            t += dt
        cuda.cuda.synchronize()
        assert t_box == t
        assert np.array_equal(_real(Ub.cpu().numpy(), ng).view(np.int64), _real(Ud.cpu().numpy(), ng).view(np.int64))
    finally:
        I.set_scheme(I.Scheme())


def test_2d_rejects_what_the_reference_2d_integrator_lacks(cuda):
    from cholla_gb300 import _lib as L
    from cholla_gb300 import integrator as I

    U = cuda.zeros((6, 1, 16, 16), dtype=cuda.float64, device="cuda")
    for scheme in (I.Scheme(riemann_solver="HLL"), I.Scheme(precision="mixed")):
        I.set_scheme(scheme)
        with pytest.raises(L.CgbError) as e:
            I.VL_Algorithm_2D_CUDA(U, 16, 16, 0, 0, 4, 0.1, 0.1, 0.0, 0.0, 1e-3, 6)
        assert e.value.code == L.CGB_ERR_UNSUPPORTED
    I.set_scheme(I.Scheme())
