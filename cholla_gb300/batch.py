"""Batches of independent 3D boxes advanced together (wrapper of the cgb_batch C ABI), and the
device initial conditions of the serving workload (blast, shock tube).

One Batch owns a job table and a CUDA stream; every job keeps its torch CUDA state tensor
resident, its own scratch, dt and time.  Batch.step(k) advances all jobs by k steps with one
chain of launches per 16 jobs (one block per tile of all of them) and one chain of the
single-box step per large job (the chains run side by side), replayed from a captured CUDA
graph; jobs can be added and removed between steps (the
graph is captured again at the next step).
"""
from __future__ import annotations

import ctypes as C

from . import _lib as L
from .integrator import Scheme, _ptr


class BatchError(L.CgbError):
    pass


def _check(rc: int) -> None:
    if rc != L.CGB_OK:
        msg = L.lib().cgb_batch_last_error()
        raise BatchError(rc, msg.decode() if msg else "")


def _stream_handle(stream) -> int:
    return 0 if stream is None else (stream if isinstance(stream, int) else stream.cuda_stream)


class Batch:
    def __init__(self, scheme: Scheme, stream, c_cfl: float = 0.3):
        self.scheme = scheme
        self.stream = stream
        self._h = C.c_void_p()
        s = scheme.to_c()
        _check(L.lib().cgb_batch_create(C.byref(self._h), C.byref(s), c_cfl, C.c_void_p(_stream_handle(stream))))

    def close(self) -> None:
        if self._h:
            L.lib().cgb_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def job_bytes(self, nx: int, ny: int, nz: int) -> int:
        return int(L.lib().cgb_batch_job_bytes(self._h, nx, ny, nz))

    def add(self, U, n_ghost: int, dx: float, dy: float, dz: float, flags=(1,) * 6, t_end: float = 0.0) -> int:
        nf, nz, ny, nx = U.shape
        fl = (C.c_int * 6)(*flags)
        jid = C.c_int()
        _check(L.lib().cgb_batch_add(self._h, _ptr(U), nx, ny, nz, n_ghost, dx, dy, dz, fl, t_end, C.byref(jid)))
        return jid.value

    def remove(self, job_id: int) -> None:
        _check(L.lib().cgb_batch_remove(self._h, job_id))

    def hold(self, job_id: int, held: bool = True) -> None:
        """Leave a job out of the steps (held) or put it back; it resumes where it stopped."""
        _check(L.lib().cgb_batch_hold(self._h, job_id, int(bool(held))))

    def set_solo_cells(self, cells: int) -> None:
        """Jobs of at least `cells` padded cells run the single-box step in a chain of their own."""
        _check(L.lib().cgb_batch_set_solo_cells(self._h, int(cells)))

    def set_chains(self, chains: int) -> None:
        """Spread the jobs over at least `chains` parallel chains of launches (same results)."""
        _check(L.lib().cgb_batch_set_chains(self._h, int(chains)))

    def set_tiles(self, tile_set: int) -> None:
        """Sweep tile set (0 or 1) of the jobs that share the batched kernels."""
        _check(L.lib().cgb_batch_set_tiles(self._h, int(tile_set)))

    def __len__(self) -> int:
        return int(L.lib().cgb_batch_n_jobs(self._h))

    def step(self, n_steps: int = 1) -> None:
        _check(L.lib().cgb_batch_step(self._h, n_steps))

    def job_time(self, job_id: int):
        """(t, last dt) of a job; raises BatchError (CGB_ERR_NONFINITE) once it has a bad cell."""
        t, dt = C.c_double(), C.c_double()
        _check(L.lib().cgb_batch_job_time(self._h, job_id, C.byref(t), C.byref(dt)))
        return t.value, dt.value

    def job_status(self, job_id: int) -> int:
        """Status bits (CGB_STATUS_*) of a job, without raising for CGB_ERR_NONFINITE."""
        f = C.c_int()
        rc = L.lib().cgb_batch_job_status(self._h, job_id, C.byref(f))
        if rc not in (L.CGB_OK, L.CGB_ERR_NONFINITE):
            _check(rc)
        return f.value


def ic_blast(U, n_ghost: int, dx: float, center, radius: float, energy: float = 1.0, rho: float = 1.0,
             p: float = 1e-5, gamma: float = 5.0 / 3.0, dual_energy: bool = True, stream=None) -> None:
    """Sedov-like blast: energy spread over the cells within radius of center (box coordinates)."""
    nf, nz, ny, nx = U.shape
    L.check(L.lib().cgb_ic_blast(_ptr(U), nx, ny, nz, n_ghost, nf, dx, dx, dx, *center, radius, energy, rho, p, gamma,
                                 int(dual_energy), C.c_void_p(_stream_handle(stream))))


def ic_shock_tube(U, n_ghost: int, dx: float, center, normal, left=(1.0, 1.0), right=(0.125, 0.1),
                  gamma: float = 5.0 / 3.0, dual_energy: bool = True, stream=None) -> None:
    """Sod tube along the unit vector `normal` through `center`: (rho, p) left and right."""
    nf, nz, ny, nx = U.shape
    L.check(L.lib().cgb_ic_shock_tube(_ptr(U), nx, ny, nz, n_ghost, nf, dx, dx, dx, *center, *normal, left[0], left[1],
                                      right[0], right[1], gamma, int(dual_energy), C.c_void_p(_stream_handle(stream))))
