"""The oracle's reconstruction building blocks against the reference's helper unit tests
(src/reconstruction/reconstruction_tests.cu), for the MHD and the hydro build (CPU only).

Inputs and fiducials come from tests/golden/reference_fiducials.json (extracted from the
reference's test source by tests/golden/extract_reference_fiducials.py); the comparison rule is
the reference's (<= 1e-14 absolute or <= 4 ULP, with the per-field absolute tolerances the
tests pass).  The PPMC-CTU helpers (Monotonize_Parabolic_Interface, Calc_Interface_Parabolic)
are not on the VL path and are not ported.
"""
import ctypes as C
import json
from pathlib import Path

import numpy as np
import pytest

from helpers import nearly_equal

GOLD = json.loads((Path(__file__).parent / "golden" / "reference_fiducials.json").read_text())
RH = GOLD["reconstruction_helpers"]
PRIM = ["density", "velocity_x", "velocity_y", "velocity_z", "pressure", "magnetic_x", "magnetic_y", "magnetic_z",
        "gas_energy"]
EIG = ["magnetosonic_speed_fast", "magnetosonic_speed_slow", "magnetosonic_speed_fast_squared",
       "magnetosonic_speed_slow_squared", "alpha_fast", "alpha_slow", "beta_y", "beta_z", "n_fs", "sign", "q_fast",
       "q_slow", "a_fast", "a_slow", "q_prime_fast", "q_prime_slow", "a_prime_fast", "a_prime_slow"]


def _prim(vals):
    out = np.zeros(9)
    out[:len(vals)] = vals
    return out


def _chr(vals):
    out = np.zeros(7)
    out[:len(vals)] = vals
    return out


def _checked(build):
    """Primitive members the reference's tests compare: Bx is the interface normal field, not
    reconstructed, so only By and Bz are checked in the MHD build."""
    return [0, 1, 2, 3, 4, 6, 7] if build == "mhd" else [0, 1, 2, 3, 4]


def _cfg(o, build, n=1, nf=None):
    mhd = build == "mhd"
    return o.config(n, n, n, 0, nf or (8 if mhd else 5), mhd=mhd)


def _assert_close(fid, got, what, tol=None):
    tol = tol or {}
    for k, (f, g) in enumerate(zip(fid, got)):
        eps = tol.get(k, 1e-14)
        assert nearly_equal(f, g, abs_eps=eps), f"{what}[{k}]: fiducial {f!r} got {g!r}"


def _sound_speed(prim, gamma):
    return np.sqrt(gamma * prim[4] / prim[0])  # hydro_utilities.h:209-212 Calc_Sound_Speed


def test_primitive_to_characteristic_mhd(oracle_lib):
    t = RH["mhd"]["tMHDReconstructionPrimitive2Characteristic"]
    st, gamma = t["structs"], t["consts"]["gamma"]
    p = _prim(st["primitive"])
    cs = _sound_speed(p, gamma)
    out = np.zeros(7)
    oracle_lib.lib().orc_t_prim_to_char(1, p, _prim(st["primitive_slope"]), np.array(st["eigenvectors"]), cs, cs * cs,
                                        out)
    _assert_close(st["fiducial_results"], out, "characteristic slope")


def test_characteristic_to_primitive_mhd(oracle_lib):
    t = RH["mhd"]["tMHDReconstructionCharacteristic2Primitive"]
    st, gamma = t["structs"], t["consts"]["gamma"]
    p = _prim(st["primitive"])
    cs = _sound_speed(p, gamma)
    out = np.zeros(9)
    oracle_lib.lib().orc_t_char_to_prim(1, p, _chr(st["characteristic_slope"]), np.array(st["eigenvectors"]), cs,
                                        cs * cs, out)
    keep = _checked("mhd")
    tol = {i: t["abs_tolerance"][PRIM[k]] for i, k in enumerate(keep) if PRIM[k] in t["abs_tolerance"]}
    assert len(tol) == 2  # velocity_y and velocity_z carry their own tolerances in the reference test
    _assert_close([st["fiducial_results"][k] for k in keep], out[keep], "primitive slope", tol)


def test_compute_eigenvectors_mhd(oracle_lib):
    t = RH["mhd"]["tMHDReconstructionComputeEigenvectors"]
    st, gamma = t["structs"], t["consts"]["gamma"]
    p = _prim(st["primitive"])
    cs = _sound_speed(p, gamma)
    out = np.zeros(18)
    oracle_lib.lib().orc_t_eigenvectors(p, cs, cs * cs, gamma, out)
    assert len(st["fiducial_results"]) == len(EIG)
    _assert_close(st["fiducial_results"], out, "eigenvectors")


@pytest.mark.parametrize("build", ["mhd", "hydro"])
def test_thread_guard(oracle_lib, build):
    t = RH[build]["tALLReconstructionThreadGuard"]
    c = t["consts"]
    n = int(c["nx"])
    cfg = _cfg(oracle_lib, build, n)
    expect = np.ones(n ** 3, dtype=int)
    for k, v in t["at"].items():
        expect[int(k)] = int(v)
    for z in range(n):
        for y in range(n):
            for x in range(n):
                got = oracle_lib.lib().orc_t_thread_guard(C.byref(cfg), int(c["order"]), x, y, z)
                assert got == expect[x + n * y + n * n * z], (x, y, z)


@pytest.mark.parametrize("build", ["mhd", "hydro"])
def test_load_data(oracle_lib, build):
    """Load_Data at the centre of a 3^3 grid holding 0, 1, 2, ... with the energy field x 500."""
    t = RH[build]["tALLReconstructionLoadData"]
    c = t["consts"]
    n, nf = int(c["nx"]), (8 if build == "mhd" else 5)
    U = np.arange(nf * n ** 3, dtype=np.float64)
    U[4 * n ** 3:5 * n ** 3] *= 5.0e2
    cfg = _cfg(oracle_lib, build, n, nf)
    cfg.gamma = c["gamma"]
    out = np.zeros(9)
    oracle_lib.lib().orc_t_load_data(C.byref(cfg), U, int(c["xid"]), int(c["yid"]), int(c["zid"]), 0, out)
    fid = t["structs"]["fiducial_data"]
    keep = list(range(len(fid)))  # Load_Data returns the cell-centred Bx too
    _assert_close([fid[k] for k in keep], out[keep], "loaded primitive")


@pytest.mark.parametrize("build", ["mhd", "hydro"])
def test_compute_slope(oracle_lib, build):
    t = RH[build]["tALLReconstructionComputeSlope"]
    st, c = t["structs"], t["consts"]
    out = np.zeros(9)
    oracle_lib.lib().orc_t_compute_slope(C.byref(_cfg(oracle_lib, build)), _prim(st["left"]), _prim(st["right"]),
                                         c["coef"], out)
    keep = _checked(build)
    _assert_close([c["fiducial_data"]] * len(keep), out[keep], "slope")


@pytest.mark.parametrize("build", ["mhd", "hydro"])
def test_van_leer_slope(oracle_lib, build):
    t = RH[build]["tALLReconstructionVanLeerSlope"]
    st = t["structs"]
    out = np.zeros(9)
    oracle_lib.lib().orc_t_van_leer_slope(C.byref(_cfg(oracle_lib, build)), _prim(st["left"]), _prim(st["right"]),
                                          out)
    keep = _checked(build)
    _assert_close([st["fiducial_data"][k] for k in keep], out[keep], "van Leer slope")


@pytest.mark.parametrize("build", ["mhd", "hydro"])
def test_monotonize_characteristic_return_primitive(oracle_lib, build):
    t = RH[build]["tALLReconstructionMonotonizeCharacteristicReturnPrimitive"]
    st, c = t["structs"], t["consts"]
    dels = [_prim(st[k]) for k in ("del_L", "del_R", "del_C", "del_G")]
    del_a = [_chr(st[k]) for k in ("del_a_L", "del_a_R", "del_a_C", "del_a_G")]
    P4 = C.c_void_p * 4
    out = np.zeros(9)
    oracle_lib.lib().orc_t_monotonize_characteristic(
        C.byref(_cfg(oracle_lib, build)), _prim(st["primitive"]), P4(*[a.ctypes.data for a in dels]),
        P4(*[a.ctypes.data for a in del_a]), np.array(st["eigenvectors"], dtype=np.float64), c["sound_speed"],
        c["sound_speed_squared"], out)
    keep = _checked(build)
    _assert_close([st["fiducial_data"][k] for k in keep], out[keep], "monotonized slope")


@pytest.mark.parametrize("build", ["mhd", "hydro"])
def test_calc_interface_linear(oracle_lib, build):
    t = RH[build]["tALLReconstructionCalcInterfaceLinear"]
    st, c = t["structs"], t["consts"]
    out = np.zeros(9)
    oracle_lib.lib().orc_t_calc_interface_linear(C.byref(_cfg(oracle_lib, build)), _prim(st["left"]),
                                                 _prim(st["right"]), c["coef"], out)
    keep = _checked(build)
    _assert_close([st["fiducial_data"][k] for k in keep], out[keep], "linear interface")


@pytest.mark.parametrize("build", ["mhd", "hydro"])
def test_write_data(oracle_lib, build):
    """Write_Data of one interface state at the centre of a 3^3 grid (zero conserved grid): the
    conserved interface values land at the fiducial offsets, everything else stays 0."""
    t = RH[build]["tALLReconstructionWriteData"]
    c = t["consts"]
    n, nf = int(c["nx"]), (8 if build == "mhd" else 5)
    cfg = _cfg(oracle_lib, build, n, nf)
    cfg.gamma = c["gamma"]
    U, Q = np.zeros(nf * n ** 3), np.zeros(nf * n ** 3)
    cid = int(c["xid"]) + n * int(c["yid"]) + n * n * int(c["zid"])
    oracle_lib.lib().orc_t_write_data(C.byref(cfg), _prim(t["structs"]["interface"]), Q, U, cid, 0)
    expect = np.zeros_like(Q)
    for k, v in t["map"].items():
        expect[int(k)] = v
    assert len(t["map"]) == (7 if build == "mhd" else 5)
    ok = nearly_equal(expect, Q)
    assert ok.all(), (np.nonzero(~ok)[0], Q[~ok], expect[~ok])


def test_plm_limit_interfaces_hydro(oracle_lib):
    t = RH["hydro"]["tHYDROReconstructionPlmLimitInterfaces"]
    f = t["fields"]
    vec = {k: _prim([f[k].get(m, 0.0) for m in PRIM]) for k in f}
    L, R = vec["interface_l_iph"].copy(), vec["interface_r_imh"].copy()
    oracle_lib.lib().orc_t_plm_limit_interfaces(C.byref(_cfg(oracle_lib, "hydro")), L, R, vec["cell_im1"],
                                                vec["cell_i"], vec["cell_ip1"])
    keep = _checked("hydro")
    _assert_close(vec["interface_l_iph_fiducial"][keep], L[keep], "l_iph")
    _assert_close(vec["interface_r_imh_fiducial"][keep], R[keep], "r_imh")
