"""ctypes binding of the reference's own VL integrators compiled as host code
(oracle/ref_host.cpp, built by oracle/build_ref_host.sh into oracle/_ref/host/<scheme>.so).

TEST INFRASTRUCTURE ONLY: tests/ run the reference itself on the CPU through this module to pin
the FP64 restatement in oracle/cholla_oracle.cpp.  The libraries exist only where the reference
source tree was present at build time; `available()` says whether one was built.
"""
from __future__ import annotations

import atexit
import ctypes as C
import shutil
import tempfile
from pathlib import Path

import numpy as np

HOST_DIR = Path(__file__).resolve().parent / "_ref" / "host"
_DP = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_libs: dict[str, C.CDLL] = {}
_tmp: Path | None = None


def path(scheme: str) -> Path:
    return HOST_DIR / f"{scheme}.so"


def available(scheme: str) -> bool:
    return path(scheme).exists()


def lib(scheme: str, shape: tuple = ()) -> C.CDLL:
    """The library of `scheme`, one loaded instance per grid shape: the reference keeps launch
    sizes in function-local statics computed on the first call (VL_3D_cuda.cu:141 and beside each
    launch), so an instance serves one shape only.  Each instance is a private copy of the file,
    because loading one path twice returns the same instance."""
    key = f"{scheme}-" + "x".join(str(int(v)) for v in shape)
    if key not in _libs:
        global _tmp
        if _tmp is None:
            _tmp = Path(tempfile.mkdtemp(prefix="ref_host_"))
            atexit.register(shutil.rmtree, _tmp, True)
        copy = _tmp / f"{key}.so"
        shutil.copyfile(path(scheme), copy)
        h = C.CDLL(str(copy))
        h.refh_set_ghost_cells.argtypes = [_DP] + [C.c_int] * 5 + [C.POINTER(C.c_int)] + [C.c_int] * 7
        h.refh_temperature_floor.argtypes = [_DP] + [C.c_int] * 5 + [C.c_double]
        h.refh_riemann.argtypes = [C.c_int, _DP, _DP, _DP] + [C.c_int] * 4 + [C.c_double, C.c_int, C.c_int]
        if hasattr(h, "refh_vl3d"):
            h.refh_vl3d.argtypes = [_DP] + [C.c_int] * 4 + [C.c_double] * 4 + [C.c_int, C.c_double, C.c_double]
            h.refh_vl2d.argtypes = [_DP] + [C.c_int] * 3 + [C.c_double] * 3 + [C.c_int, C.c_double]
            h.refh_vl1d.argtypes = [_DP, C.c_int, C.c_int, C.c_double, C.c_double, C.c_int, C.c_double]
        for name in ("refh_plmp", "refh_ppmp"):
            getattr(h, name).argtypes = [_DP, _DP, _DP] + [C.c_int] * 4 + [C.c_double] * 3 + [C.c_int] * 2
        _libs[key] = h
    return _libs[key]


def _check(rc: int, what: str) -> None:
    if rc != 0:
        raise RuntimeError(f"reference {what} failed ({rc})")


def vl_step_3d(scheme: str, U: np.ndarray, nx, ny, nz, n_ghost, dx, dy, dz, dt, gamma, density_floor=0.0) -> None:
    """VL_Algorithm_3D_CUDA (integrators/VL_3D_cuda.cu:38) on the flat field-major state U."""
    _check(lib(scheme, (nx, ny, nz)).refh_vl3d(U, nx, ny, nz, n_ghost, dx, dy, dz, dt, U.size // (nx * ny * nz), gamma,
                                 density_floor), "VL 3D step")


def vl_step_2d(scheme: str, U: np.ndarray, nx, ny, n_ghost, dx, dy, dt, gamma) -> None:
    """VL_Algorithm_2D_CUDA (integrators/VL_2D_cuda.cu:25)."""
    _check(lib(scheme, (nx, ny)).refh_vl2d(U, nx, ny, n_ghost, dx, dy, dt, U.size // (nx * ny), gamma), "VL 2D step")


def vl_step_1d(scheme: str, U: np.ndarray, nx, n_ghost, dx, dt, gamma) -> None:
    """VL_Algorithm_1D_CUDA (integrators/VL_1D_cuda.cu:30)."""
    _check(lib(scheme, (nx,)).refh_vl1d(U, nx, n_ghost, dx, dt, U.size // nx, gamma), "VL 1D step")


def riemann(scheme: str, solver: int, QL: np.ndarray, QR: np.ndarray, F: np.ndarray, nx, ny, nz, n_ghost, gamma,
            direction) -> None:
    """One launch of a flux kernel (0 HLLC, 1 Roe, 3 HLL, 4 exact) along `direction`."""
    _check(lib(scheme, (nx, ny, nz)).refh_riemann(solver, QL, QR, F, nx, ny, nz, n_ghost, gamma, direction,
                                                  QL.size // (nx * ny * nz)), "Riemann solver")


def set_boundaries(scheme: str, U: np.ndarray, nx, ny, nz, n_ghost, flags) -> None:
    """Grid3D::Set_Boundaries_Grid's ghost fill: SetGhostCells for faces 0-5 in turn
    (grid/boundary_conditions.cpp:104-116), over the ghost slabs of Set_Boundary_Extents
    (:419-493), on the faces whose axis has more than one cell."""
    h = lib(scheme, (nx, ny, nz))
    fl = (C.c_int * 6)(*flags)
    jl, ju = (n_ghost, ny - n_ghost) if ny > 1 else (0, ny)
    kl, ku = (n_ghost, nz - n_ghost) if nz > 1 else (0, nz)
    slabs = [((0, n_ghost), (jl, ju), (kl, ku)), ((nx - n_ghost, nx), (jl, ju), (kl, ku)),
             ((0, nx), (0, n_ghost), (kl, ku)), ((0, nx), (ny - n_ghost, ny), (kl, ku)),
             ((0, nx), (0, ny), (0, n_ghost)), ((0, nx), (0, ny), (nz - n_ghost, nz))]
    for face, ext in enumerate((nx, nx, ny, ny, nz, nz)):
        if ext <= 1:
            continue
        (i0, i1), (j0, j1), (k0, k1) = slabs[face]
        _check(h.refh_set_ghost_cells(U, nx, ny, nz, U.size // (nx * ny * nz), n_ghost, fl, i1 - i0, j1 - j0, k1 - k0,
                                      i0, j0, k0, face), "ghost fill")


def temperature_floor(scheme: str, U: np.ndarray, nx, ny, nz, n_ghost, U_floor) -> None:
    """Apply_Temperature_Floor (hydro/hydro_cuda.cu:1103)."""
    _check(lib(scheme, (nx, ny, nz)).refh_temperature_floor(U, nx, ny, nz, n_ghost, U.size // (nx * ny * nz),
                                                            U_floor), "temperature floor")


def reconstruct(scheme: str, kind: str, U: np.ndarray, QL: np.ndarray, QR: np.ndarray, nx, ny, nz, n_ghost, dx, dt,
                gamma, direction) -> None:
    """One launch of PLMP_cuda or PPMP_cuda (kind "plmp" / "ppmp") along `direction`."""
    h = lib(scheme, (nx, ny, nz))
    fn = h.refh_plmp if kind == "plmp" else h.refh_ppmp
    _check(fn(U, QL, QR, nx, ny, nz, n_ghost, dx, dt, gamma, direction, U.size // (nx * ny * nz)), kind)
