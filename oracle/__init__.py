"""ctypes binding of the FP64 CPU oracle (oracle/cholla_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and bench.py's CPU
baseline.  The cholla_gb300 package never imports this module.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIBPATH = HERE / "_build" / "libcholla_oracle.so"

PCM, PLMC, PPMC, PLMP, PPMP = 0, 1, 2, 3, 4
HLLC, ROE, HLLD, HLL, EXACT = 0, 1, 2, 3, 4


class orc_config(C.Structure):
    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("n_ghost", C.c_int), ("n_fields", C.c_int),
        ("n_scalars", C.c_int), ("de", C.c_int), ("mhd", C.c_int), ("recon", C.c_int), ("solver", C.c_int),
        ("density_floor_on", C.c_int), ("gamma", C.c_double), ("dx", C.c_double), ("dy", C.c_double),
        ("dz", C.c_double), ("density_floor", C.c_double),
    ]


_lib = None
_DP = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")


def build() -> Path:
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIBPATH


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIBPATH.exists():
            build()
        h = C.CDLL(str(LIBPATH))
        P = C.POINTER(orc_config)
        sig = {
            "orc_pcm_3d": [P, _DP, _DP, _DP, _DP, _DP, _DP, _DP],
            "orc_ppmc_vl": [P, _DP, _DP, _DP, C.c_int],
            "orc_plmc": [P, _DP, _DP, _DP, C.c_int],
            "orc_plmp": [P, _DP, _DP, _DP, C.c_int],
            "orc_ppmp": [P, _DP, _DP, _DP, C.c_int],
            "orc_hllc": [P, _DP, _DP, _DP, C.c_int],
            "orc_roe": [P, _DP, _DP, _DP, C.c_int],
            "orc_hlld": [P, _DP, _DP, _DP, _DP, C.c_int],
            "orc_hll": [P, _DP, _DP, _DP, C.c_int],
            "orc_exact": [P, _DP, _DP, _DP, C.c_int],
            "orc_ct_electric_fields": [P, _DP, _DP, _DP, _DP, _DP],
            "orc_update_magnetic": [P, _DP, _DP, _DP, C.c_double],
            "orc_update_half": [P, _DP, _DP, _DP, _DP, _DP, C.c_double],
            "orc_de_partial_update": [P, _DP, C.c_double],
            "orc_update_full": [P, _DP, _DP, _DP, _DP, C.c_double],
            "orc_de_select": [P, _DP],
            "orc_de_sync": [P, _DP],
            "orc_temperature_floor": [P, _DP, C.c_double],
            "orc_set_boundaries": [P, _DP, C.POINTER(C.c_int)],
            "orc_vl_step_3d": [P, _DP, C.c_double],
            "orc_vl_step_1d": [P, _DP, C.c_double],
            "orc_vl_step_2d": [P, _DP, C.c_double],
            "orc_mt19937_uniform": [C.c_ulonglong, C.c_double, C.c_double, C.c_size_t, _DP],
            "orc_mt19937_32_uniform": [C.c_ulong, C.c_double, C.c_double, C.c_size_t, _DP],
            "orc_ppm_single_variable": [C.c_double] * 5 + [C.POINTER(C.c_double)] * 2,
            "orc_set_threads": [C.c_int],
            "orc_t_load_data": [P, _DP, C.c_int, C.c_int, C.c_int, C.c_int, _DP],
            "orc_t_write_data": [P, _DP, _DP, _DP, C.c_size_t, C.c_int],
            "orc_t_compute_slope": [P, _DP, _DP, C.c_double, _DP],
            "orc_t_van_leer_slope": [P, _DP, _DP, _DP],
            "orc_t_eigenvectors": [_DP, C.c_double, C.c_double, C.c_double, _DP],
            "orc_t_prim_to_char": [C.c_int, _DP, _DP, _DP, C.c_double, C.c_double, _DP],
            "orc_t_char_to_prim": [C.c_int, _DP, _DP, _DP, C.c_double, C.c_double, _DP],
            "orc_t_monotonize_characteristic": [P, _DP, C.c_void_p * 4, C.c_void_p * 4, _DP, C.c_double, C.c_double,
                                                _DP],
            "orc_t_calc_interface_linear": [P, _DP, _DP, C.c_double, _DP],
            "orc_t_plm_limit_interfaces": [P, _DP, _DP, _DP, _DP, _DP],
            "orc_t_cell_centered_b": [_DP, C.c_size_t, C.c_int, C.c_int, C.c_int, C.c_size_t, C.c_int, C.c_int,
                                      C.c_int, _DP],
            "orc_t_hlld_load_state": [P, _DP, C.c_double, C.c_size_t, C.c_int, _DP],
            "orc_t_hlld_return_fluxes": [P, C.c_size_t, C.c_int, _DP, _DP, _DP],
            "orc_t_hlld_lr_speeds": [_DP, _DP, C.c_double, C.c_double, _DP],
            "orc_t_hlld_nonstar_fluxes": [_DP, C.c_double, _DP],
            "orc_t_hlld_star_state": [_DP, _DP, C.c_double, C.c_double, C.c_double, _DP],
            "orc_t_hlld_star_fluxes": [_DP, _DP, _DP, _DP, C.c_double, _DP],
            "orc_t_hlld_double_star_state": [_DP, _DP, C.c_double, C.c_double, _DP, _DP],
            "orc_t_hlld_double_star_fluxes": [_DP, C.c_double, _DP, _DP, _DP, _DP, C.c_double, C.c_double, _DP],
        }
        for name, args in sig.items():
            getattr(h, name).argtypes = args
            getattr(h, name).restype = C.c_int if name.startswith("orc_vl_step") else None
        h.orc_calc_dt.argtypes = [P, _DP]
        h.orc_calc_dt.restype = C.c_double
        h.orc_t_thread_guard.argtypes = [P, C.c_int, C.c_int, C.c_int, C.c_int]
        h.orc_t_thread_guard.restype = C.c_int
        D = C.c_double
        for name, args in (("orc_t_pressure_primitive", [D] * 6 + [C.c_int] + [D] * 3),
                           ("orc_t_energy_primitive", [D] * 6 + [C.c_int] + [D] * 3),
                           ("orc_t_pressure_from_de", [D] * 4), ("orc_t_kinetic_energy", [D] * 4),
                           ("orc_t_magnetic_energy", [D] * 3), ("orc_t_total_pressure", [D] * 4),
                           ("orc_t_fast_magnetosonic", [D] * 6), ("orc_t_slow_magnetosonic", [D] * 6),
                           ("orc_t_alfven_speed", [D] * 2),
                           ("orc_t_hlld_middle_speed", [_DP, _DP, _DP]),
                           ("orc_t_hlld_star_speed", [_DP, _DP, C.c_double, C.c_double]),
                           ("orc_t_hlld_star_total_pressure", [_DP, _DP, _DP])):
            getattr(h, name).argtypes = args
            getattr(h, name).restype = C.c_double
        h.orc_ct_slope.argtypes = [P, _DP, _DP, C.c_double] + [C.c_int] * 8
        h.orc_ct_slope.restype = C.c_double
        h.orc_max_divB.argtypes = [P, _DP]
        h.orc_max_divB.restype = C.c_double
        h.orc_get_threads.restype = C.c_int
        _lib = h
    return _lib


def config(nx, ny, nz, n_ghost, n_fields, *, n_scalars=0, de=False, mhd=False, recon=PPMC, solver=HLLC,
           density_floor_on=True, gamma=5.0 / 3.0, dx=1.0, dy=1.0, dz=1.0, density_floor=0.0) -> orc_config:
    return orc_config(nx, ny, nz, n_ghost, n_fields, n_scalars, int(de), int(mhd), recon, solver,
                      int(density_floor_on), gamma, dx, dy, dz, density_floor)


def mt_uniform(seed: int, a: float, b: float, n: int) -> np.ndarray:
    out = np.empty(n, dtype=np.float64)
    lib().orc_mt19937_uniform(seed, a, b, n, out)
    return out


def mt32_uniform(seed: int, a: float, b: float, n: int) -> np.ndarray:
    out = np.empty(n, dtype=np.float64)
    lib().orc_mt19937_32_uniform(seed, a, b, n, out)
    return out


def vl_step_3d(cfg: orc_config, U: np.ndarray, dt: float) -> None:
    rc = lib().orc_vl_step_3d(C.byref(cfg), U, dt)
    if rc != 0:
        raise ValueError("oracle rejected the configuration")


def vl_step_1d(cfg: orc_config, U: np.ndarray, dt: float) -> None:
    rc = lib().orc_vl_step_1d(C.byref(cfg), U, dt)
    if rc != 0:
        raise ValueError("oracle rejected the configuration")


def vl_step_2d(cfg: orc_config, U: np.ndarray, dt: float) -> None:
    rc = lib().orc_vl_step_2d(C.byref(cfg), U, dt)
    if rc != 0:
        raise ValueError("oracle rejected the configuration")


def calc_dt(cfg: orc_config, U: np.ndarray) -> float:
    return lib().orc_calc_dt(C.byref(cfg), U)


def set_boundaries(cfg: orc_config, U: np.ndarray, flags) -> None:
    arr = (C.c_int * 6)(*flags)
    lib().orc_set_boundaries(C.byref(cfg), U, arr)


def temperature_floor(cfg: orc_config, U: np.ndarray, U_floor: float) -> None:
    lib().orc_temperature_floor(C.byref(cfg), U, U_floor)


def set_threads(n: int) -> None:
    lib().orc_set_threads(n)


def get_threads() -> int:
    return lib().orc_get_threads()
