"""ctypes binding of oracle/ref_harness.cpp: the reference's own CUDA kernels, compiled from
the cholla source tree into oracle/_ref/<variant>/*.cubin by oracle/build_ref.sh.

TEST INFRASTRUCTURE ONLY (parity against the reference's own build on the same GPU, and
the speed of that build).  Variants: hydro_ppmc_hllc_de, hydro_ppmc_hllc, hydro_plmc_hllc,
hydro_ppmc_roe_de, mhd_plmc_hlld.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

HERE = Path(__file__).resolve().parent
REF_DIR = HERE / "_ref"
LIBPATH = HERE / "_build" / "libref_harness.so"

_lib = None
_variant = None


def available(variant: str = "hydro_ppmc_hllc_de") -> bool:
    return (REF_DIR / variant).is_dir() and any((REF_DIR / variant).glob("*.cubin"))


def _load() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIBPATH.exists():
            import subprocess

            subprocess.run(["make", "-s", "-C", str(HERE), "ref"], check=True)
        h = C.CDLL(str(LIBPATH))
        U, I, D = C.c_ulonglong, C.c_int, C.c_double
        h.refh_error.restype = C.c_char_p
        h.refh_init.argtypes = [C.c_char_p, C.c_char_p]
        h.refh_set_stream.argtypes = [C.c_void_p]
        h.refh_vl_step_3d.argtypes = [U, I, I, I, I, D, D, D, D, I, D, D]
        h.refh_vl_step_1d.argtypes = [U, I, I, D, D, I, D]
        h.refh_calc_dt.argtypes = [U, I, I, I, I, I, D, D, D, D, C.POINTER(D)]
        h.refh_temperature_floor.argtypes = [U, I, I, I, I, I, D]
        h.refh_set_boundaries.argtypes = [U, I, I, I, I, I, C.POINTER(I)]
        h.refh_set_sync_each.argtypes = [I]
        _lib = h
    return _lib


def _check(rc: int) -> None:
    if rc != 0:
        raise RuntimeError("reference harness: " + _load().refh_error().decode())


def init(variant: str) -> None:
    global _variant
    h = _load()
    if _variant != variant:
        _check(h.refh_init(str(REF_DIR / variant).encode(), variant.encode()))
        _variant = variant


def set_stream(stream) -> None:
    _load().refh_set_stream(C.c_void_p(0 if stream is None else stream.cuda_stream))


def vl_step_3d(U, nx, ny, nz, ng, dx, dy, dz, dt, nf, gamma, density_floor=0.0) -> None:
    _check(_load().refh_vl_step_3d(U.data_ptr(), nx, ny, nz, ng, dx, dy, dz, dt, nf, gamma, density_floor))


def vl_step_1d(U, nx, ng, dx, dt, nf, gamma) -> None:
    _check(_load().refh_vl_step_1d(U.data_ptr(), nx, ng, dx, dt, nf, gamma))


def calc_dt(U, nx, ny, nz, ng, nf, dx, dy, dz, gamma) -> float:
    out = C.c_double()
    _check(_load().refh_calc_dt(U.data_ptr(), nx, ny, nz, ng, nf, dx, dy, dz, gamma, C.byref(out)))
    return out.value


def temperature_floor(U, nx, ny, nz, ng, nf, U_floor) -> None:
    _check(_load().refh_temperature_floor(U.data_ptr(), nx, ny, nz, ng, nf, U_floor))


def set_boundaries(U, nx, ny, nz, ng, nf, flags) -> None:
    arr = (C.c_int * 6)(*flags)
    _check(_load().refh_set_boundaries(U.data_ptr(), nx, ny, nz, ng, nf, arr))


def sync() -> None:
    _check(_load().refh_sync())


def set_sync_each(on: bool) -> None:
    """Synchronise after every kernel (the reference's default build, src/utils/gpu.hpp:139-155) or
    not (its -DDISABLE_GPU_ERROR_CHECKING build, the default here)."""
    _check(_load().refh_set_sync_each(int(bool(on))))
