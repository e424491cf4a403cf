"""The oracle's hydro and MHD utility functions that the VL step calls, against the reference's
utility unit tests (src/utils/hydro_utilities_tests.cpp, src/utils/mhd_utilities_tests.cu),
for the MHD and the hydro build where the fiducials differ (CPU only).

Parameters and fiducials come from tests/golden/reference_fiducials.json.  The comparison rule
is the reference's (<= 1e-14 absolute or <= 4 ULP); as in the reference, the absolute part
makes the tiny-number cases pass on magnitude alone.  The floors are checked for exact
equality with TINY_NUMBER, as the reference does.  Utilities the step does not call
(Calc_Pressure_Conserved, Calc_Energy_Conserved, Calc_Temp, Calc_Temp_DE,
Calc_Kinetic_Energy_From_Momentum, computeThermalEnergy, the vector-potential initialiser) are
not ported.
"""
import json
from pathlib import Path

import numpy as np
import pytest

from helpers import nearly_equal

U = json.loads((Path(__file__).parent / "golden" / "reference_fiducials.json").read_text())["utilities"]
TINY = 1e-20
BUILDS = ["mhd", "hydro"]


def _hydro(build):
    d = U["hydro_utilities"][build]
    return d["params"], d["tests"]


def _mhd():
    d = U["mhd_utilities"]["mhd"]
    return d["params"], d["tests"]


def _cases(p):
    return range(len(p["d"] if "d" in p else p["density"]))


@pytest.mark.parametrize("build", BUILDS)
def test_calc_pressure_primitive(oracle_lib, build):
    p, t = _hydro(build)
    fid = t["tHYDROtMHDHydroUtilsCalcPressurePrimitive.CorrectInputExpectCorrectOutput"]["vectors"]["fiducial_pressure"]
    L = oracle_lib.lib()
    for i in _cases(p):
        got = L.orc_t_pressure_primitive(p["E"][i], p["d"][i], p["vx"][i], p["vy"][i], p["vz"][i], p["gamma"],
                                         int(build == "mhd"), p["magnetic_x"][i], p["magnetic_y"][i],
                                         p["magnetic_z"][i])
        assert nearly_equal(fid[i], got), (i, got, fid[i])
        # NegativePressureExpectAutomaticFix: x velocity scaled by 1e4 gives exactly TINY_NUMBER
        neg = L.orc_t_pressure_primitive(p["E"][i], p["d"][i], 1e4 * p["vx"][i], p["vy"][i], p["vz"][i],
                                         p["gamma"], int(build == "mhd"), p["magnetic_x"][i], p["magnetic_y"][i],
                                         p["magnetic_z"][i])
        assert neg == TINY, (i, neg)


@pytest.mark.parametrize("build", BUILDS)
@pytest.mark.parametrize("kind", ["CorrectInputExpectCorrectOutput", "NegativePressureExpectAutomaticFix"])
def test_calc_energy_primitive(oracle_lib, build, kind):
    p, t = _hydro(build)
    fid = t[f"tHYDROtMHDHydroUtilsCalcEnergyPrimitive.{kind}"]["vectors"]["fiducial_energy"]
    sign = -1.0 if kind.startswith("Negative") else 1.0
    for i in _cases(p):
        got = oracle_lib.lib().orc_t_energy_primitive(sign * p["P"][i], p["d"][i], p["vx"][i], p["vy"][i],
                                                      p["vz"][i], p["gamma"], int(build == "mhd"),
                                                      p["magnetic_x"][i], p["magnetic_y"][i], p["magnetic_z"][i])
        assert nearly_equal(fid[i], got), (i, got, fid[i])


def test_get_pressure_from_de(oracle_lib):
    p, t = _hydro("hydro")
    fid = t["tHYDROHydroUtilsGetPressureFromDE.CorrectInputExpectCorrectOutput"]["vectors"]["fiducial_Ps"]
    for i in _cases(p):
        got = oracle_lib.lib().orc_t_pressure_from_de(p["E"][i], p["U_total"][i], p["U_advected"][i], p["gamma"])
        assert nearly_equal(fid[i], got), (i, got, fid[i])


def test_kinetic_energy_from_velocity(oracle_lib):
    p, t = _hydro("hydro")
    case = t["tHYDROtMHDCalcKineticEnergyFromVelocity.CorrectInputExpectCorrectOutput"]
    c, fid = case["coef"], case["vectors"]["fiducialEnergies"]
    for i in _cases(p):
        got = oracle_lib.lib().orc_t_kinetic_energy(c * p["d"][i], c * p["vx"][i], c * p["vy"][i], c * p["vz"][i])
        assert nearly_equal(fid[i], got), (i, got, fid[i])


def test_magnetic_energy(oracle_lib):
    p, t = _mhd()
    fid = t["tMHDcomputeMagneticEnergy.CorrectInputExpectCorrectOutput"]["vectors"]["fiducialEnergy"]
    for i in _cases(p):
        got = oracle_lib.lib().orc_t_magnetic_energy(p["magneticX"][i], p["magneticY"][i], p["magneticZ"][i])
        assert nearly_equal(fid[i], got), (i, got, fid[i])


def test_total_pressure(oracle_lib):
    p, t = _mhd()
    fid = t["tMHDComputeTotalPressure.CorrectInputExpectCorrectOutput"]["vectors"]["fiducialTotalPressures"]
    mult = t["tMHDComputeTotalPressure.NegativePressureExpectAutomaticFix"]["vectors"]["pressureMultiplier"]
    L = oracle_lib.lib()
    for i in _cases(p):
        b = (p["magneticX"][i], p["magneticY"][i], p["magneticZ"][i])
        got = L.orc_t_total_pressure(p["pressureGas"][i], *b)
        assert nearly_equal(fid[i], got), (i, got, fid[i])
        assert L.orc_t_total_pressure(mult[i] * p["pressureGas"][i], *b) == TINY, i


@pytest.mark.parametrize("kind,sign", [("CorrectInputExpectCorrectOutput", 1.0),
                                       ("NegativeDensityExpectAutomaticFix", -1.0)])
def test_fast_magnetosonic_speed(oracle_lib, kind, sign):
    p, t = _mhd()
    v = t[f"tMHDFastMagnetosonicSpeed.{kind}"]["vectors"]
    fid, coef = v["fiducialFastMagnetosonicSpeed"], v["coef"]
    for i in _cases(p):
        c = coef[i]
        got = oracle_lib.lib().orc_t_fast_magnetosonic(sign * c * p["density"][i], c * p["pressureGas"][i],
                                                       c * p["magneticX"][i], c * p["magneticY"][i],
                                                       c * p["magneticZ"][i], p["gamma"])
        assert nearly_equal(fid[i], got), (i, got, fid[i])


@pytest.mark.parametrize("kind,sign", [("CorrectInputExpectCorrectOutput", 1.0),
                                       ("NegativeDensityExpectAutomaticFix", -1.0)])
def test_slow_magnetosonic_speed(oracle_lib, kind, sign):
    p, t = _mhd()
    case = t[f"tMHDSlowMagnetosonicSpeed.{kind}"]
    fid, c = case["vectors"]["fiducialSlowMagnetosonicSpeed"], case["coef"]
    assert case["start"] == 2  # the reference checks the large-number case only
    for i in range(case["start"], len(fid)):
        got = oracle_lib.lib().orc_t_slow_magnetosonic(sign * p["density"][i] * c, p["pressureGas"][i] * c,
                                                       p["magneticX"][i] * c, p["magneticY"][i] * c,
                                                       p["magneticZ"][i] * c, p["gamma"])
        assert nearly_equal(fid[i], got), (i, got, fid[i])


@pytest.mark.parametrize("kind,sign", [("CorrectInputExpectCorrectOutput", 1.0),
                                       ("NegativeDensityExpectAutomaticFix", -1.0)])
def test_alfven_speed(oracle_lib, kind, sign):
    p, t = _mhd()
    fid = t[f"tMHDAlfvenSpeed.{kind}"]["vectors"]["fiducialAlfvenSpeed"]
    for i in _cases(p):
        got = oracle_lib.lib().orc_t_alfven_speed(p["magneticX"][i], sign * p["density"][i])
        assert nearly_equal(fid[i], got), (i, got, fid[i])


def test_cell_centered_magnetic_fields(oracle_lib):
    """cellCenteredMagneticFields at (1, 1, 1) of a grid with 3 x 3 strides, 125 cells per field
    and 8 fields holding 0, 1, 2, ... (magnetic_x is field 5)."""
    _, t = _mhd()
    c = t["tMHDCellCenteredMagneticFields.CorrectInputExpectCorrectOutput"]["consts"]
    nx, ny, n_cells = int(c["nx"]), int(c["ny"]), 5 ** 3
    x = nx // 2
    cid = x + x * nx + x * nx * ny
    grid = np.arange(n_cells * 8, dtype=np.float64)
    out = np.zeros(3)
    oracle_lib.lib().orc_t_cell_centered_b(grid, cid, x, x, x, n_cells, nx, ny, 5, out)
    assert nearly_equal(np.array([c["fiducialAvgBx"], c["fiducialAvgBy"], c["fiducialAvgBz"]]), out).all(), out
