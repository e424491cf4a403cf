"""Host-side mirror of the reference's integrator interface, over the libchollagb C ABI.

Function names, argument order and meaning follow the reference
(src/integrators/VL_3D_cuda.h:9-13, src/integrators/VL_1D_cuda.h, src/hydro/hydro_cuda.h:69-70,
src/grid/boundary_conditions.cpp).  Device arrays are torch CUDA tensors (float64, contiguous,
field-major) or raw device addresses (int).  Errors raise CgbError instead of aborting.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

from . import _lib as L


def _ptr(a) -> int:
    if a is None:
        return 0
    if isinstance(a, int):
        return a
    if not a.is_cuda:
        raise L.CgbError(L.CGB_ERR_ARGS, "device array expected (torch CUDA tensor)")
    if not a.is_contiguous():
        raise L.CgbError(L.CGB_ERR_ARGS, "array must be contiguous")
    import torch

    if a.dtype != torch.float64:
        raise L.CgbError(L.CGB_ERR_ARGS, "state must be float64")
    return a.data_ptr()


_RECON = {"PCM": L.PCM, "PLMC": L.PLMC, "PPMC": L.PPMC, "PLMP": L.PLMP, "PPMP": L.PPMP}
_SOLVER = {"HLLC": L.HLLC, "ROE": L.ROE, "HLLD": L.HLLD, "HLL": L.HLL, "EXACT": L.EXACT}
_PREC = {"fp64": L.FP64, "mixed": L.MIXED, "fp64_fast": L.FP64_FAST}


@dataclass
class Scheme:
    """The reference's make.type choices plus `gama`, as run-time options."""

    reconstruction: str = "PPMC"
    riemann_solver: str = "HLLC"
    dual_energy: bool = True
    mhd: bool = False
    n_scalars: int = 0
    density_floor: bool = True
    temperature_floor: bool = True
    precision: str = "fp64"
    gamma: float = 5.0 / 3.0
    U_floor: float = 0.0

    @property
    def n_fields(self) -> int:
        return 5 + self.n_scalars + (3 if self.mhd else 0) + (1 if self.dual_energy else 0)

    def n_ghost(self) -> int:
        """Ghost layers the reference uses for this scheme (src/grid/grid3D.cpp:53-76)."""
        g = {"PCM": 2, "PLMC": 3, "PPMC": 4, "PLMP": 3, "PPMP": 4}[self.reconstruction]
        return g + (1 if self.mhd else 0)

    def to_c(self) -> L.cgb_scheme:
        return L.cgb_scheme(
            _RECON[self.reconstruction], _SOLVER[self.riemann_solver], int(self.dual_energy), int(self.mhd),
            int(self.n_scalars), int(self.density_floor), int(self.temperature_floor), _PREC[self.precision],
            float(self.gamma), float(self.U_floor))


def set_scheme(scheme: Scheme) -> None:
    s = scheme.to_c()
    L.check(L.lib().cgb_set_scheme(C.byref(s)))


def get_scheme() -> L.cgb_scheme:
    s = L.cgb_scheme()
    L.check(L.lib().cgb_get_scheme(C.byref(s)))
    return s


def set_stream(stream) -> None:
    """Queue subsequent calls on a torch.cuda.Stream (or a raw cudaStream_t / None)."""
    handle = 0 if stream is None else (stream if isinstance(stream, int) else stream.cuda_stream)
    L.check(L.lib().cgb_set_stream(C.c_void_p(handle)))


def VL_Algorithm_3D_CUDA(d_conserved, d_grav_potential, nx, ny, nz, x_off, y_off, z_off, n_ghost, dx, dy, dz,
                         xbound, ybound, zbound, dt, n_fields, custom_grav, density_floor,
                         host_grav_potential=None) -> None:
    L.check(L.lib().cgb_vl_algorithm_3d(
        _ptr(d_conserved), _ptr(d_grav_potential), nx, ny, nz, x_off, y_off, z_off, n_ghost, dx, dy, dz, xbound,
        ybound, zbound, dt, n_fields, custom_grav, density_floor,
        None if host_grav_potential is None else host_grav_potential))


def VL_Algorithm_1D_CUDA(d_conserved, nx, x_off, n_ghost, dx, xbound, dt, n_fields, custom_grav=0) -> None:
    L.check(L.lib().cgb_vl_algorithm_1d(_ptr(d_conserved), nx, x_off, n_ghost, dx, xbound, dt, n_fields,
                                        custom_grav))


def VL_Algorithm_2D_CUDA(d_conserved, nx, ny, x_off, y_off, n_ghost, dx, dy, xbound, ybound, dt, n_fields,
                         custom_grav=0) -> None:
    L.check(L.lib().cgb_vl_algorithm_2d(_ptr(d_conserved), nx, ny, x_off, y_off, n_ghost, dx, dy, xbound, ybound,
                                        dt, n_fields, custom_grav))


def Free_Memory_VL_3D() -> None:
    L.check(L.lib().cgb_free_memory_vl_3d())


def Calc_dt_GPU(dev_conserved, nx, ny, nz, n_ghost, n_fields, dx, dy, dz, gamma) -> float:
    """Maximum inverse crossing time over the real cells (the host computes dt = C_cfl / value)."""
    out = C.c_double(0.0)
    L.check(L.lib().cgb_calc_dt_gpu(_ptr(dev_conserved), nx, ny, nz, n_ghost, n_fields, dx, dy, dz, gamma,
                                    C.byref(out)))
    return out.value


def Apply_Temperature_Floor(dev_conserved, nx, ny, nz, n_ghost, n_fields, U_floor) -> None:
    L.check(L.lib().cgb_apply_temperature_floor(_ptr(dev_conserved), nx, ny, nz, n_ghost, n_fields, U_floor))


def Set_Boundaries(dev_conserved, nx, ny, nz, n_ghost, n_fields, flags) -> None:
    """Fill every ghost cell.  flags = (xl, xu, yl, yu, zl, zu): 1 periodic, 2 reflective,
    3 transmissive, 4 custom (untouched)."""
    arr = (C.c_int * 6)(*[int(f) for f in flags])
    L.check(L.lib().cgb_set_boundaries(_ptr(dev_conserved), nx, ny, nz, n_ghost, n_fields, arr))


def Max_Magnetic_Divergence(dev_conserved, nx, ny, nz, n_ghost, n_fields, dx, dy, dz) -> float:
    """Max |div B| of an MHD state over the cells with x, y, z >= 2, upper ghost layers included,
    as the reference's kernel measures it (src/mhd/magnetic_divergence.cu:33-105): fill the ghost
    cells first."""
    out = C.c_double(0.0)
    L.check(L.lib().cgb_max_magnetic_divergence(_ptr(dev_conserved), nx, ny, nz, n_ghost, n_fields, dx, dy, dz,
                                                C.byref(out)))
    return out.value


def Check_Magnetic_Divergence(dev_conserved, nx, ny, nz, n_ghost, n_fields, dx, dy, dz) -> float:
    """checkMagneticDivergence (src/mhd/magnetic_divergence.cu:92-120): the maximum |div B|, raising
    CgbError with CGB_ERR_NONFINITE where the reference would exit (above 1e-9, negative or NaN)."""
    out = C.c_double(0.0)
    rc = L.lib().cgb_check_magnetic_divergence(_ptr(dev_conserved), nx, ny, nz, n_ghost, n_fields, dx, dy, dz,
                                               C.byref(out))
    L.check(rc)
    return out.value


def Check_Status() -> int:
    """Status bits (CGB_STATUS_*) the drop-in steps collected since the last call, which clears
    them; raises CgbError (CGB_ERR_NONFINITE) when a real cell went non-finite.  The reference
    prints such cells from the device (src/hydro/hydro_cuda.cu:381-389)."""
    f = C.c_int(0)
    L.check(L.lib().cgb_check_status(C.byref(f)))
    return f.value


def debug_fail_alloc(n: int) -> None:
    """Make the n-th device allocation of the library from now on fail (0: off).  Test hook."""
    L.check(L.lib().cgb_debug_fail_alloc(int(n)))
