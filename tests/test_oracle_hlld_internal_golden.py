"""The oracle's HLLD building blocks against the reference's HLLD-internal unit tests
(src/riemann_solvers/hlld_cuda_tests.cu:1811-2400, the mhd::internal functions), CPU only.

The shared test parameters (two cases of states, star states, fluxes and wave speeds) and the
fiducials come from tests/golden/reference_fiducials.json; states are packed in the member
order of mhd::internal::State (9), StarState (6), DoubleStarState (6), Flux (7) and Speeds (5).
Comparison rule: the reference's (<= 1e-14 absolute or <= 4 ULP, with the per-field absolute
tolerances the tests pass).
"""
import ctypes as C
import json
from pathlib import Path

import numpy as np
import pytest

from helpers import nearly_equal

GOLD = json.loads((Path(__file__).parent / "golden" / "reference_fiducials.json").read_text())["hlld_internal"]
P = GOLD["params"]
T = GOLD["tests"]
FLUX = ["density", "momentumX", "momentumY", "momentumZ", "energy", "magneticY", "magneticZ"]
STAR = ["density", "velocityY", "velocityZ", "energy", "magneticY", "magneticZ"]
DSTAR = ["velocityY", "velocityZ", "magneticY", "magneticZ", "energyL", "energyR"]
STATE = ["density", "velocityX", "velocityY", "velocityZ", "energy", "magneticY", "magneticZ", "gasPressure",
         "totalPressure"]
CASES = range(len(P["magneticX"]))


def _a(v):
    return np.ascontiguousarray(v, dtype=np.float64)


def _check(fid, got, names, test, case, skip=()):
    tol = test["abs_tolerance"]
    for k, name in enumerate(names):
        if name in skip:
            continue
        assert nearly_equal(fid[k], got[k], abs_eps=tol.get(name, 1e-14)), \
            f"case {case} {name}: fiducial {fid[k]!r} got {got[k]!r}"


def test_approximate_lr_wave_speeds(oracle_lib):
    t = T["tMHDHlldInternalApproximateLRWaveSpeeds.CorrectInputExpectCorrectOutput"]
    for i in CASES:
        sp = np.zeros(5)
        oracle_lib.lib().orc_t_hlld_lr_speeds(_a(P["stateLVec"][i]), _a(P["stateRVec"][i]), P["magneticX"][i],
                                              P["gamma"], sp)
        assert nearly_equal(t["fiducial"]["fiducialSpeedL"][i], sp[0]), (i, sp)
        assert nearly_equal(t["fiducial"]["fiducialSpeedR"][i], sp[4]), (i, sp)


def test_approximate_middle_wave_speed(oracle_lib):
    t = T["tMHDHlldInternalApproximateMiddleWaveSpeed.CorrectInputExpectCorrectOutput"]
    for i in CASES:
        got = oracle_lib.lib().orc_t_hlld_middle_speed(_a(P["stateLVec"][i]), _a(P["stateRVec"][i]), _a(P["speed"][i]))
        assert nearly_equal(t["fiducial"]["fiducialSpeedM"][i], got), (i, got)


def test_approximate_star_wave_speed(oracle_lib):
    t = T["tMHDHlldInternalApproximateStarWaveSpeed.CorrectInputExpectCorrectOutput"]
    L = oracle_lib.lib()
    for i in CASES:
        sl = L.orc_t_hlld_star_speed(_a(P["starStateLVec"][i]), _a(P["speed"][i]), P["magneticX"][i], -1.0)
        sr = L.orc_t_hlld_star_speed(_a(P["starStateRVec"][i]), _a(P["speed"][i]), P["magneticX"][i], 1.0)
        assert nearly_equal(t["fiducial"]["fiducialSpeedStarL"][i], sl), (i, sl)
        assert nearly_equal(t["fiducial"]["fiducialSpeedStarR"][i], sr), (i, sr)


def test_non_star_fluxes(oracle_lib):
    t = T["tMHDHlldInternalNonStarFluxes.CorrectInputExpectCorrectOutput"]
    for i in CASES:
        f = np.zeros(7)
        oracle_lib.lib().orc_t_hlld_nonstar_fluxes(_a(P["stateLVec"][i]), P["magneticX"][i], f)
        _check(t["fiducial"]["fiducialFlux"][i], f, FLUX, t, i)


@pytest.mark.parametrize("kind", ["NonDegenerate", "Degenerate"])
def test_compute_star_state(oracle_lib, kind):
    t = T[f"tMHDHlldInternalComputeStarState.CorrectInput{kind}ExpectCorrectOutput"]
    states = [list(s) for s in P["stateLVec"]]
    if t["multiplier"]:
        states[0][8] *= t["multiplier"]  # the degenerate test scales case 0's total pressure
    for i in CASES:
        st = np.zeros(6)
        speed = _a(P["speed"][i])
        oracle_lib.lib().orc_t_hlld_star_state(_a(states[i]), speed, speed[0], P["magneticX"][i],
                                               P["totalPressureStar"][i], st)
        _check(t["fiducial"]["fiducialStarState"][i], st, STAR, t, i, skip=("density",))


def test_star_fluxes_non_degenerate(oracle_lib):
    t = T["tMHDHlldInternalStarFluxes.CorrectInputNonDegenerateExpectCorrectOutput"]
    L = oracle_lib.lib()
    for i in CASES:
        speed = _a(P["speed"][i])
        st, f = np.zeros(6), np.zeros(7)
        L.orc_t_hlld_star_state(_a(P["stateLVec"][i]), speed, speed[0], P["magneticX"][i], P["totalPressureStar"][i],
                                st)
        L.orc_t_hlld_star_fluxes(st, _a(P["stateLVec"][i]), _a(P["flux"][i]), speed, speed[0], f)
        _check(t["fiducial"]["fiducialFlux"][i], f, FLUX, t, i)


def test_star_fluxes_degenerate(oracle_lib):
    t = T["tMHDHlldInternalStarFluxes.CorrectInputDegenerateExpectCorrectOutput"]
    for i in CASES:
        speed = _a(P["speed"][i])
        f = np.zeros(7)
        oracle_lib.lib().orc_t_hlld_star_fluxes(_a(P["starStateLVec"][i]), _a(P["stateLVec"][i]), _a(P["flux"][i]),
                                                speed, speed[0], f)
        _check(t["fiducial"]["fiducialFlux"][i], f, FLUX, t, i)


@pytest.mark.parametrize("kind", ["NonDegenerate", "Degenerate"])
def test_double_star_state(oracle_lib, kind):
    t = T[f"tMHDHlldInternalDoubleStarState.CorrectInput{kind}ExpectCorrectOutput"]
    for i in CASES:
        out = np.zeros(6)
        bx = P["magneticX"][i] if kind == "NonDegenerate" else 0.0
        oracle_lib.lib().orc_t_hlld_double_star_state(_a(P["starStateLVec"][i]), _a(P["starStateRVec"][i]), bx,
                                                      P["totalPressureStar"][i], _a(P["speed"][i]), out)
        _check(t["fiducial"]["fiducialState"][i], out, DSTAR, t, i)


def test_double_star_fluxes(oracle_lib):
    t = T["tMHDHlldInternalDoubleStarFluxes.CorrectInputExpectCorrectOutput"]
    for i in CASES:
        speed = _a(P["speed"][i])
        ds = _a(P["DoubleStarStateVec"][i])
        f = np.zeros(7)
        oracle_lib.lib().orc_t_hlld_double_star_fluxes(ds, ds[4], _a(P["starStateLVec"][i]), _a(P["stateLVec"][i]),
                                                       _a(P["flux"][i]), speed, speed[0], speed[1], f)
        _check(t["fiducial"]["fiducialFlux"][i], f, FLUX, t, i)


def test_return_fluxes(oracle_lib):
    """returnFluxes writes the seven flux members to the x-direction's fields of cell 0 and
    touches nothing else (10 cells x 8 fields pre-filled with a dummy value)."""
    t = T["tMHDHlldInternalReturnFluxes.CorrectInputExpectCorrectOutput"]
    n, nf = 10, 8
    cfg = oracle_lib.config(n, 1, 1, 0, nf, mhd=True)
    F = np.full(n * nf, t["dummy"])
    oracle_lib.lib().orc_t_hlld_return_fluxes(C.byref(cfg), 0, 0, F, _a(t["flux"]), _a(t["state"]))
    # density, momenta x/y/z, energy, then By and Bz into the magnetic_x / magnetic_y slots
    where = [0, n * 1, n * 2, n * 3, n * 4, n * 5, n * 6]
    expect = np.full(n * nf, t["dummy"])
    expect[where] = t["flux"]
    assert np.array_equal(F, expect), np.nonzero(F != expect)


def test_star_total_pressure(oracle_lib):
    t = T["tMHDHlldInternalStarTotalPressure.CorrectInputExpectCorrectOutput"]
    for i in CASES:
        got = oracle_lib.lib().orc_t_hlld_star_total_pressure(_a(P["stateLVec"][i]), _a(P["stateRVec"][i]),
                                                              _a(P["speed"][i]))
        assert nearly_equal(t["fiducial"]["fiducialPressure"][i], got), (i, got)


def test_load_state(oracle_lib):
    """loadState from an interface array holding 1, 2, 3, ... (10 cells x 8 fields) in each of
    the three directions."""
    t = T["tMHDHlldInternalLoadState.CorrectInputExpectCorrectOutput"]
    n, nf = t["n_cells"], 8
    cfg = oracle_lib.config(n, 1, 1, 0, nf, mhd=True, gamma=P["gamma"])
    Q = np.arange(1, n * nf + 1, dtype=np.float64)
    for d in range(3):
        out = np.zeros(9)
        oracle_lib.lib().orc_t_hlld_load_state(C.byref(cfg), Q, P["magneticX"][0], 0, d, out)
        _check(t["fiducial"]["fiducialState"][d], out, STATE, t, d)
