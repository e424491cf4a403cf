"""The reference's MHD linear-wave system test run through the oracle (CPU only), with the
reference MHD build's scheme (PLMC + HLLD + CT, builds/make.type.mhd): the fast magnetosonic
wave along x on 64 x 32 x 32 cells for one crossing of the box
(src/system_tests/mhd_system_tests.cpp:125-161).  The step count the reference expects, each
field's L1 change (face fields over the faces the reference writes out), the norm of the L1
vector and the largest change within the reference's PLMC bounds.  The other waves and
directions run on the GPU (tests/test_system_mhd_waves_gpu.py); through the oracle they take
minutes.
"""
import json
from pathlib import Path

import numpy as np
import pytest

from helpers import l1_errors_mhd, mhd_wave_state, run_reference_loop

SYS = json.loads((Path(__file__).parent / "golden" / "reference_fiducials.json").read_text())["mhd_system"]


def test_fast_magnetosonic_wave_oracle(oracle_lib):
    o = oracle_lib
    name = "FastMagnetosonicWaveRightMovingCorrectInputExpectCorrectOutput"
    case, angle, ng = SYS["tests"][name], SYS["angles"][0], 4
    U, (Nx, Ny, Nz), dx, tout = mhd_wave_state(SYS, case, angle, ng)
    cfg = o.config(Nx, Ny, Nz, ng, 8, mhd=True, recon=o.PLMC, solver=o.HLLD, gamma=SYS["gamma"], dx=dx, dy=dx, dz=dx)
    U = np.ascontiguousarray(U.ravel())
    o.set_boundaries(cfg, U, (1,) * 6)
    U0 = U.copy()
    n, t = run_reference_loop(lambda dt: o.vl_step_3d(cfg, U, dt), lambda: o.calc_dt(cfg, U),
                              lambda: o.set_boundaries(cfg, U, (1,) * 6), tout)
    assert n == case["n_steps"][0] and t == tout, (n, t)
    l1, norm, worst = l1_errors_mhd(U0.reshape(8, Nz, Ny, Nx), U.reshape(8, Nz, Ny, Nx), ng)
    max_l1, max_error = case["bounds"]["PLMC"]
    assert (l1 < max_l1).all() and norm < max_l1 and worst < max_error, (l1, norm, worst)


def test_constant_states_oracle(oracle_lib):
    """The MHD constant-state system tests (mhd_system_tests.cpp:710-722), 16^3 with and
    without a field, PLMC + HLLD, to t = 1e5: every real cell and face keeps its initial value
    bit for bit (the reference compares with data files that can hold nothing else)."""
    from helpers import constant_state, real_slice

    o = oracle_lib
    cs = json.loads((Path(__file__).parent / "golden" / "reference_fiducials.json").read_text())["constant_states"]
    for key in ("mhd_field", "mhd_zero_field"):
        st, ng = cs[key]["settings"], 4
        U, (Nx, Ny, Nz), dx = constant_state(st, ng, mhd=True)
        cfg = o.config(Nx, Ny, Nz, ng, 8, mhd=True, recon=o.PLMC, solver=o.HLLD, gamma=st["gamma"], dx=dx, dy=dx,
                       dz=dx)
        U = np.ascontiguousarray(U.ravel())
        U0 = U.copy()
        o.set_boundaries(cfg, U, (1,) * 6)
        n, t = run_reference_loop(lambda dt: o.vl_step_3d(cfg, U, dt), lambda: o.calc_dt(cfg, U),
                                  lambda: o.set_boundaries(cfg, U, (1,) * 6), st["tout"])
        assert t == st["tout"] and n > 10, (key, n, t)
        R = U.reshape(8, Nz, Ny, Nx)[real_slice(ng)]
        R0 = U0.reshape(8, Nz, Ny, Nx)[real_slice(ng)]
        assert np.array_equal(R.view(np.int64), R0.view(np.int64)), key



@pytest.mark.parametrize("di", [1, 2], ids=["y", "z"])
def test_fast_wave_low_resolution_rotated_oracle(oracle_lib, di):
    """The N = 16 fast wave of the convergence test along y (yaw = pi/2) and z (pitch = pi/2):
    the reference's step count for that direction and its bounds for the low-resolution run
    (mhd_system_tests.cpp:391-425), checking the rotated initial condition on the CPU."""
    o = oracle_lib
    case, angle, ng = SYS["tests"]["FastMagnetosonicWaveExpectSecondOrderConvergence"], SYS["angles"][di], 4
    U, (Nx, Ny, Nz), dx, tout = mhd_wave_state(SYS, case, angle, ng)
    cfg = o.config(Nx, Ny, Nz, ng, 8, mhd=True, recon=o.PLMC, solver=o.HLLD, gamma=SYS["gamma"], dx=dx, dy=dx, dz=dx)
    U = np.ascontiguousarray(U.ravel())
    o.set_boundaries(cfg, U, (1,) * 6)
    U0 = U.copy()
    n, t = run_reference_loop(lambda dt: o.vl_step_3d(cfg, U, dt), lambda: o.calc_dt(cfg, U),
                              lambda: o.set_boundaries(cfg, U, (1,) * 6), tout)
    assert n == case["n_steps"][di] and t == tout, (n, t)
    l1, norm, worst = l1_errors_mhd(U0.reshape(8, Nz, Ny, Nx), U.reshape(8, Nz, Ny, Nx), ng)
    max_l1, max_error = case["bounds"]["PLMC"]
    assert (l1 < max_l1).all() and norm < max_l1 and worst < max_error, (l1, norm, worst)
