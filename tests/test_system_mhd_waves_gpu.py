"""The reference's MHD linear-wave system tests through libchollagb on the GPU
(src/system_tests/mhd_system_tests.cpp:30-541), HLLD + constrained transport:

* fast, slow and Alfven waves in both directions and the contact wave, each along x, y and z
  (the reference's pitch / yaw / domain / direction tuples), 64 x 32 x 32 cells for one
  crossing, driven like the reference's main loop through the drop-in C ABI (exact FP64):
  the reference's step count per direction, each field's L1 change (face fields over the
  faces the reference writes out), the norm of the L1 vector and the largest change within
  the bounds for the reconstruction.  PLMC (the reference MHD build's) along all three
  directions, PCM and PPMC along x;
* second-order convergence: the N = 16 run's L1 norm is 4 +- 0.2 times the N = 32 one (PLMC);
* the box engine (dt on the device, clamped to the output time) in exact and fast FP64.
"""
import json
from pathlib import Path

import numpy as np
import pytest

from helpers import l1_errors_mhd, mhd_wave_state, run_reference_loop

pytestmark = pytest.mark.gpu

SYS = json.loads((Path(__file__).parent / "golden" / "reference_fiducials.json").read_text())["mhd_system"]
NG = {"PCM": 3, "PLMC": 4, "PPMC": 5}
WAVES = [n for n in SYS["tests"] if "Convergence" not in n]
CONVERGENCE = [n for n in SYS["tests"] if "Convergence" in n]
BY_KEY = {SYS["tests"][n]["key"]: n for n in WAVES if SYS["tests"][n].get("key")}


def _scheme(recon, precision="fp64", gamma=SYS["gamma"]):
    from cholla_gb300 import integrator as I

    return I.Scheme(reconstruction=recon, riemann_solver="HLLD", mhd=True, dual_energy=False, gamma=gamma,
                    precision=precision)


def _dropin(cuda, name, recon, di, N=None):
    """Run one case through the drop-in C ABI; returns (steps, final time, tout, L1, norm, max)."""
    from cholla_gb300 import integrator as I

    case = SYS["tests"][name]
    ng = NG[recon]
    U, (Nx, Ny, Nz), dx, tout = mhd_wave_state(SYS, case, SYS["angles"][di], ng, N)
    I.set_scheme(_scheme(recon))
    G = cuda.from_numpy(U).cuda()
    fill = lambda: I.Set_Boundaries(G, Nx, Ny, Nz, ng, 8, (1,) * 6)  # noqa: E731
    fill()
    U0 = G.cpu().numpy()
    n, t = run_reference_loop(
        lambda dt: I.VL_Algorithm_3D_CUDA(G, None, Nx, Ny, Nz, 0, 0, 0, ng, dx, dx, dx, 0, 0, 0, dt, 8, 0, 0.0),
        lambda: I.Calc_dt_GPU(G, Nx, Ny, Nz, ng, 8, dx, dx, dx, SYS["gamma"]), fill, tout)
    return (n, t, tout, *l1_errors_mhd(U0, G.cpu().numpy(), ng))


def _check(case, recon, di, res):
    n, t, tout, l1, norm, worst = res
    max_l1, max_error = case["bounds"][recon]
    assert n == case["n_steps"][di] and t == tout, (n, case["n_steps"][di], t, tout)
    assert (l1 < max_l1).all(), (l1, max_l1)
    assert norm < max_l1 and worst < max_error, (norm, worst, max_l1, max_error)


CASES = [(name, "PLMC", di) for di in range(3) for name in WAVES] + \
        [(name, recon, 0) for recon in ("PCM", "PPMC") for name in WAVES]


@pytest.mark.parametrize("name,recon,di", CASES, ids=[f"{n[:-len('CorrectInputExpectCorrectOutput')]}-{r}-"
                                                      f"{'xyz'[d]}" for n, r, d in CASES])
def test_mhd_linear_wave_dropin_exact(cuda, name, recon, di):
    _check(SYS["tests"][name], recon, di, _dropin(cuda, name, recon, di))


@pytest.mark.parametrize("di", range(3), ids=list("xyz"))
@pytest.mark.parametrize("name", CONVERGENCE)
def test_mhd_linear_wave_second_order(cuda, name, di):
    """The N = 16 run meets its own bounds, and its L1 norm over the N = 32 run's is 4 +- 0.2."""
    case = SYS["tests"][name]
    low = _dropin(cuda, name, "PLMC", di)
    _check(case, "PLMC", di, low)
    conv = case["convergence"]
    high = _dropin(cuda, BY_KEY[conv["of"]], "PLMC", di)
    ratio = low[4] / high[4]
    assert abs(ratio - conv["ratio"]) <= conv["tolerance"], ratio


@pytest.mark.parametrize("precision", ["fp64", "fp64_fast"])
@pytest.mark.parametrize("name", [WAVES[0], WAVES[4], WAVES[6]],
                         ids=["fast", "alfven", "contact"])
def test_mhd_linear_wave_box_engine(cuda, precision, name):
    """Box engine along x, PLMC: after the reference's step count less one the time is short
    of the output time, after one more it is there, and the bounds hold."""
    from cholla_gb300.engine import Box

    case, recon, di = SYS["tests"][name], "PLMC", 0
    ng = NG[recon]
    U, (Nx, Ny, Nz), dx, tout = mhd_wave_state(SYS, case, SYS["angles"][di], ng)
    G = cuda.from_numpy(U.copy()).cuda()
    from cholla_gb300 import integrator as I

    I.set_scheme(_scheme(recon))
    I.Set_Boundaries(G, Nx, Ny, Nz, ng, 8, (1,) * 6)
    U0 = G.cpu().numpy()
    box = Box(Nx, Ny, Nz, ng, dx, dx, dx, _scheme(recon, precision))
    try:
        box.set_time(0.0, tout)
        box.advance(G, case["n_steps"][di] - 1)
        t_before, _ = box.time()
        box.advance(G, 1)
        t_end, _ = box.time()
    finally:
        box.close()
    assert t_before < tout and t_end == tout, (t_before, t_end, tout)
    l1, norm, worst = l1_errors_mhd(U0, G.cpu().numpy(), ng)
    max_l1, max_error = case["bounds"][recon]
    assert (l1 < max_l1).all() and norm < max_l1 and worst < max_error, (l1, norm, worst)


CONST = json.loads((Path(__file__).parent / "golden" / "reference_fiducials.json").read_text())["constant_states"]


@pytest.mark.parametrize("precision", ["fp64", "fp64_fast"])
@pytest.mark.parametrize("key", ["mhd_field", "mhd_zero_field"])
def test_mhd_constant_state(cuda, key, precision):
    """mhd_system_tests.cpp:710-722 (16^3, PLMC + HLLD, to t = 1e5), exact through the drop-in
    C ABI and fast through the box engine: every real cell and face keeps its value bit for
    bit."""
    from cholla_gb300 import integrator as I
    from cholla_gb300.engine import Box
    from helpers import constant_state, real_slice

    st, recon = CONST[key]["settings"], "PLMC"
    ng = NG[recon]
    U, (Nx, Ny, Nz), dx = constant_state(st, ng, mhd=True)
    G = cuda.from_numpy(U.copy()).cuda()
    if precision == "fp64":
        I.set_scheme(_scheme(recon, gamma=st["gamma"]))
        fill = lambda: I.Set_Boundaries(G, Nx, Ny, Nz, ng, 8, (1,) * 6)  # noqa: E731
        fill()
        n, t = run_reference_loop(
            lambda dt: I.VL_Algorithm_3D_CUDA(G, None, Nx, Ny, Nz, 0, 0, 0, ng, dx, dx, dx, 0, 0, 0, dt, 8, 0, 0.0),
            lambda: I.Calc_dt_GPU(G, Nx, Ny, Nz, ng, 8, dx, dx, dx, st["gamma"]), fill, st["tout"])
    else:
        box = Box(Nx, Ny, Nz, ng, dx, dx, dx, _scheme(recon, precision, st["gamma"]))
        try:
            box.set_time(0.0, st["tout"])
            t, n = 0.0, 0
            while t < st["tout"] and n < 5000:
                box.advance(G, 1)
                t, _ = box.time()
                n += 1
        finally:
            box.close()
    assert t == st["tout"] and n > 10, (t, n)
    rs = real_slice(ng)
    assert np.array_equal(G.cpu().numpy()[rs].view(np.int64), U[rs].view(np.int64))
