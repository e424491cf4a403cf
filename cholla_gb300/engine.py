"""Device-resident time stepping of one box (wrapper of the cgb_box C ABI).

A Box owns the scratch of one padded grid and advances a torch CUDA state tensor in place:
ghost fill, dt = C_cfl / max inverse crossing time (on the device), VL step, temperature
floor and the CFL reduction for the next step -- the body of the reference's main loop
(src/main.cpp:247-379) without a host round trip per step.
"""
from __future__ import annotations

import ctypes as C

from . import _lib as L
from .integrator import Scheme, _ptr


class BoxError(L.CgbError):
    pass


def _check(rc: int) -> None:
    if rc != L.CGB_OK:
        msg = L.lib().cgb_box_last_error()
        raise BoxError(rc, msg.decode() if msg else "")


class Box:
    def __init__(self, nx: int, ny: int, nz: int, n_ghost: int, dx: float, dy: float, dz: float, scheme: Scheme,
                 flags=(1, 1, 1, 1, 1, 1)):
        self.shape = (nx, ny, nz)
        self.n_ghost = n_ghost
        self.scheme = scheme
        self._h = C.c_void_p()
        s = scheme.to_c()
        fl = (C.c_int * 6)(*flags)
        _check(L.lib().cgb_box_create(C.byref(self._h), nx, ny, nz, n_ghost, dx, dy, dz, C.byref(s), fl))
        self.n_fields = L.lib().cgb_box_n_fields(self._h)

    def close(self) -> None:
        if self._h:
            L.lib().cgb_box_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_time(self, t: float, t_end: float = 0.0) -> None:
        _check(L.lib().cgb_box_set_time(self._h, t, t_end))

    def use_graph(self, enable: bool = True) -> None:
        _check(L.lib().cgb_box_use_graph(self._h, int(enable)))

    def enable_timing(self, enable: bool = True) -> None:
        _check(L.lib().cgb_box_enable_timing(self._h, int(enable)))

    def kernel_times(self):
        ms = (C.c_double * 3)()
        n = C.c_longlong()
        _check(L.lib().cgb_box_kernel_times(self._h, ms, C.byref(n)))
        return {"predictor": ms[0], "corrector": ms[1], "finalize": ms[2], "steps": n.value}

    def advance(self, U, n_steps: int = 1, c_cfl: float = 0.3, stream=None) -> None:
        handle = 0 if stream is None else (stream if isinstance(stream, int) else stream.cuda_stream)
        _check(L.lib().cgb_box_advance(self._h, _ptr(U), n_steps, c_cfl, C.c_void_p(handle)))

    def time(self):
        """(t, last dt); raises BoxError with code CGB_ERR_NONFINITE once a step has left a bad cell."""
        t = C.c_double()
        dt = C.c_double()
        _check(L.lib().cgb_box_get_time(self._h, C.byref(t), C.byref(dt)))
        return t.value, dt.value

    def check_status(self) -> int:
        """Status bits (CGB_STATUS_*) of the steps since the last call, which clears them; raises
        BoxError (CGB_ERR_NONFINITE) when a real cell went non-finite."""
        f = C.c_int()
        _check(L.lib().cgb_box_check_status(self._h, C.byref(f)))
        return f.value
