"""The throughput arithmetic paths against the oracle, by tolerance (they are not bit-exact).

fast FP64 (CGB_FP64_FAST): relative L1 error of every field <= 1e-12 after one step and after
20 steps of the turbulence box.  Mixed precision (CGB_MIXED): relative L1 density error <= 1e-5
after 20 steps (the accuracy target of the mixed-precision form), per-field errors printed.
Relative L1 = sum|gpu - oracle| / sum|oracle| over real cells.
"""
import numpy as np
import pytest

from helpers import real_slice

pytestmark = pytest.mark.gpu

FIELDS = ["density", "momentum_x", "momentum_y", "momentum_z", "Energy", "GasEnergy"]


def rel_l1(got, want, ng):
    g, w = got[real_slice(ng)], want[real_slice(ng)]
    return np.abs(g - w).sum(axis=(1, 2, 3)) / np.abs(w).sum(axis=(1, 2, 3))


def _run_pair(cuda, oracle_lib, U0, ng, scheme, steps, dx):
    from cholla_gb300 import integrator as I

    o = oracle_lib
    nf, nz, ny, nx = U0.shape
    I.set_scheme(scheme)
    Ug = cuda.from_numpy(U0.copy()).cuda()
    Uo = U0.copy()
    cfg = o.config(nx, ny, nz, ng, nf, de=scheme.dual_energy, n_scalars=scheme.n_scalars,
                   recon=getattr(o, scheme.reconstruction),
                   solver=getattr(o, scheme.riemann_solver), gamma=scheme.gamma,
                   dx=dx[0], dy=dx[1], dz=dx[2])
    for _ in range(steps):
        dt = 0.3 / o.calc_dt(cfg, Uo.reshape(-1))  # same dt sequence for both (the oracle's)
        I.VL_Algorithm_3D_CUDA(Ug, None, nx, ny, nz, 0, 0, 0, ng, *dx, 0, 0, 0, dt, nf, 0, 0.0)
        I.Set_Boundaries(Ug, nx, ny, nz, ng, nf, (1,) * 6)
        o.vl_step_3d(cfg, Uo.reshape(-1), dt)
        o.set_boundaries(cfg, Uo.reshape(-1), (1,) * 6)
    return Ug.cpu().numpy(), Uo


@pytest.mark.parametrize("recon", ["PCM", "PLMC", "PPMC", "PLMP", "PPMP"])
@pytest.mark.parametrize("solver", ["HLLC", "ROE", "HLL"])
def test_fast_fp64_one_step(cuda, oracle_lib, recon, solver):
    from cholla_gb300 import ics
    from cholla_gb300 import integrator as I

    ng = {"PCM": 2, "PLMC": 3, "PPMC": 4, "PLMP": 3, "PPMP": 4}[recon]
    U0 = ics.smooth_random_box((19, 13, 11), ng, np.random.default_rng(7), dual_energy=True)
    s = I.Scheme(reconstruction=recon, riemann_solver=solver, dual_energy=True, precision="fp64_fast")
    got, want = _run_pair(cuda, oracle_lib, U0, ng, s, 1, (1 / 19, 1 / 13, 1 / 11))
    err = rel_l1(got, want, ng)
    assert np.all(err <= 1e-12), dict(zip(FIELDS, err))


@pytest.mark.parametrize("precision,tol", [("fp64_fast", 1e-12), ("mixed", 1e-5)])
def test_hll_with_scalars_five_steps(cuda, oracle_lib, precision, tol):
    """HLL in the throughput forms with two passive scalars and dual energy, 5 steps against the
    oracle: every field within 1e-12 relative L1 (fast FP64), density within 1e-5 (mixed)."""
    from cholla_gb300 import ics
    from cholla_gb300 import integrator as I

    ng = 4
    U0 = ics.smooth_random_box((17, 14, 12), ng, np.random.default_rng(11), dual_energy=True, n_scalars=2)
    s = I.Scheme(reconstruction="PPMC", riemann_solver="HLL", dual_energy=True, n_scalars=2, precision=precision)
    got, want = _run_pair(cuda, oracle_lib, U0, ng, s, 5, (1 / 17, 1 / 14, 1 / 12))
    err = rel_l1(got, want, ng)
    names = FIELDS[:5] + ["scalar_0", "scalar_1", "GasEnergy"]
    print(precision, {f: f"{e:.2e}" for f, e in zip(names, err)})
    assert np.isfinite(got).all()
    assert np.all(err <= tol) if precision == "fp64_fast" else err[0] <= tol, dict(zip(names, err))


@pytest.mark.parametrize("recon", ["PLMC", "PPMC", "PPMP"])
@pytest.mark.parametrize("precision", ["fp64_fast", "mixed"])
def test_exact_solver_in_the_throughput_forms(cuda, oracle_lib, recon, precision):
    """The exact Riemann solver in the throughput forms, 5 steps against the oracle.  The reference
    evaluates its fractional powers with single-precision powf, which CUDA and the host's libm may
    round one binary32 ulp apart (the exact FP64 form is held to 1e-7 for the same reason): every
    field within 1e-7 relative L1 in fast FP64, density within 1e-5 in mixed."""
    from cholla_gb300 import ics
    from cholla_gb300 import integrator as I

    ng = {"PLMC": 3, "PPMC": 4, "PPMP": 4}[recon]
    U0 = ics.smooth_random_box((17, 14, 12), ng, np.random.default_rng(13), dual_energy=True)
    s = I.Scheme(reconstruction=recon, riemann_solver="EXACT", dual_energy=True, precision=precision)
    got, want = _run_pair(cuda, oracle_lib, U0, ng, s, 5, (1 / 17, 1 / 14, 1 / 12))
    err = rel_l1(got, want, ng)
    print(precision, recon, {f: f"{e:.2e}" for f, e in zip(FIELDS, err)})
    assert np.isfinite(got).all()
    assert np.all(err <= 1e-7) if precision == "fp64_fast" else err[0] <= 1e-5, dict(zip(FIELDS, err))


def test_fast_fp64_turbulence_20_steps(cuda, oracle_lib):
    """20 steps of the rms-Mach-2 turbulence box: every field within 1e-12 relative L1."""
    from cholla_gb300 import ics
    from cholla_gb300 import integrator as I

    n, ng = 32, 4
    U0 = ics.turbulence_box(n, ng, 5 / 3, seed=4)
    s = I.Scheme(reconstruction="PPMC", riemann_solver="HLLC", dual_energy=True, precision="fp64_fast")
    got, want = _run_pair(cuda, oracle_lib, U0, ng, s, 20, (1 / n,) * 3)
    err = rel_l1(got, want, ng)
    print("fp64_fast", {f: f"{e:.2e}" for f, e in zip(FIELDS, err)})
    assert np.isfinite(got).all()
    assert np.all(err <= 1e-12), dict(zip(FIELDS, err))


@pytest.mark.parametrize("seed,mach,solver,recon", [(4, 2.0, "HLLC", "PPMC"), (6, 3.0, "HLLC", "PPMC"),
                                                    (4, 2.0, "HLL", "PPMC"), (4, 2.0, "HLLC", "PPMP"),
                                                    (6, 3.0, "ROE", "PLMP")])
def test_mixed_turbulence_20_steps(cuda, oracle_lib, seed, mach, solver, recon):
    """Mixed precision, 20 steps of rms-Mach-2 and -3 turbulence boxes: finite everywhere and
    relative L1 density error <= 1e-5 (the accuracy target of the mixed-precision form)."""
    from cholla_gb300 import ics
    from cholla_gb300 import integrator as I

    n, ng = 32, 4
    U0 = ics.turbulence_box(n, ng, 5 / 3, seed=seed, mach=mach)
    s = I.Scheme(reconstruction=recon, riemann_solver=solver, dual_energy=True, precision="mixed")
    got, want = _run_pair(cuda, oracle_lib, U0, ng, s, 20, (1 / n,) * 3)
    err = rel_l1(got, want, ng)
    print(f"mixed {recon} {solver} seed {seed} mach {mach}", {f: f"{e:.2e}" for f, e in zip(FIELDS, err)})
    assert np.isfinite(got).all()
    assert err[0] <= 1e-5, dict(zip(FIELDS, err))


def test_engine_matches_dropin_sequence_bitwise(cuda):
    """The box engine (device-side dt, fused floor + CFL reduction, CUDA-graph replay) gives
    the same state, bit for bit, as the drop-in call sequence of the reference's main loop."""
    from cholla_gb300 import ics
    from cholla_gb300 import integrator as I
    from cholla_gb300.engine import Box

    n, ng, gamma = 32, 4, 5 / 3
    U0 = ics.turbulence_box(n, ng, gamma, seed=6)
    nf, N = U0.shape[0], U0.shape[1]
    dx = 1 / n
    s = I.Scheme(reconstruction="PPMC", riemann_solver="HLLC", dual_energy=True, temperature_floor=True)
    I.set_scheme(s)
    Ua = cuda.from_numpy(U0.copy()).cuda()
    for _ in range(6):
        I.Set_Boundaries(Ua, N, N, N, ng, nf, (1,) * 6)
        dt = 0.3 / I.Calc_dt_GPU(Ua, N, N, N, ng, nf, dx, dx, dx, gamma)
        I.VL_Algorithm_3D_CUDA(Ua, None, N, N, N, 0, 0, 0, ng, dx, dx, dx, 0, 0, 0, dt, nf, 0, 0.0)
        I.Apply_Temperature_Floor(Ua, N, N, N, ng, nf, 0.0)
    stream = cuda.cuda.Stream()
    for graph in (False, True):
        Ub = cuda.from_numpy(U0.copy()).cuda()
        box = Box(N, N, N, ng, dx, dx, dx, s)
        box.use_graph(graph)
        box.advance(Ub, 6, 0.3, stream)
        stream.synchronize()
        t, dt_last = box.time()
        a, b = Ua.cpu().numpy()[real_slice(ng)], Ub.cpu().numpy()[real_slice(ng)]
        assert (a.view(np.int64) == b.view(np.int64)).all(), f"graph={graph}"
        assert t > 0 and dt_last > 0
        box.close()


@pytest.mark.parametrize("precision,ns,flags", [("mixed", 0, (1,) * 6), ("fp64_fast", 0, (1,) * 6),
                                                ("mixed", 1, (2, 3, 1, 1, 3, 2)), ("fp64_fast", 2, (3, 2, 2, 3, 1, 1))])
def test_engine_carried_primitives_bitwise(cuda, precision, ns, flags):
    """Within one advance call the mixed form's finalize writes the next step's primitives of the
    real cells and the next step forms only the ghosts' (the state is the engine's between its
    steps); every call starts from primitives of all cells.  Six steps in one call equal six
    one-step calls bit for bit, with passive scalars and reflective / outflow faces, whose ghosts
    are not copies (the fast FP64 form, which forms all primitives every step, runs the same check)."""
    from cholla_gb300 import ics
    from cholla_gb300 import integrator as I
    from cholla_gb300.engine import Box

    n, ng, gamma = 24, 4, 5 / 3
    rng = np.random.default_rng(8)
    U0 = ics.smooth_random_box((n, n, n), ng, rng, dual_energy=True, n_scalars=ns)
    N = U0.shape[1]
    dx = 1 / n
    s = I.Scheme(reconstruction="PPMC", riemann_solver="HLLC", dual_energy=True, n_scalars=ns,
                 temperature_floor=True, precision=precision)
    stream = cuda.cuda.Stream()
    out = []
    for calls in (1, 6):
        U = cuda.from_numpy(U0.copy()).cuda()
        box = Box(N, N, N, ng, dx, dx, dx, s, flags=flags)
        box.use_graph(True)
        for _ in range(calls):
            box.advance(U, 6 // calls, 0.3, stream)
        stream.synchronize()
        out.append((U.cpu().numpy(), box.time()))
        box.close()
    (a, ta), (b, tb) = out
    rs = real_slice(ng)
    assert np.array_equal(a[rs].view(np.int64), b[rs].view(np.int64))
    assert ta == tb
