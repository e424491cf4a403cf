"""cgb_vl_algorithm_3d_static: the VL step with its scratch in the library's static device pool.

The file name makes pytest collect it last; it also passes when run alone.  The step must
match the allocating entry point, cgb_vl_algorithm_3d, over two calls in a row, leave the
device's free memory unchanged once the first call on the device has located the pool, and
reject a box larger than the pool with a message.
"""
import ctypes

import numpy as np
import pytest

from helpers import real_slice

pytestmark = pytest.mark.gpu

PRECISIONS = {"fp64": 0.0, "fp64_fast": 1e-12, "mixed": 1e-6}  # relative L1 tolerance per field


def _static_step(lib, U, N, ng, dx, dt, nf):
    return lib.cgb_vl_algorithm_3d_static(ctypes.c_void_p(U.data_ptr()), None, N, N, N, 0, 0, 0, ng, dx, dx, dx, 0.0,
                                          0.0, 0.0, dt, nf, 0, 0.0, None)


@pytest.mark.parametrize("precision", list(PRECISIONS))
def test_static_step_matches_allocating_step_twice(cuda, precision):
    from cholla_gb300 import _lib, ics
    from cholla_gb300 import integrator as I

    lib = _lib.lib()
    n, ng = 32, 4
    U0 = ics.turbulence_box(n, ng, 5 / 3, seed=8)
    nf, N = U0.shape[0], U0.shape[1]
    dx = 1 / n
    I.set_scheme(I.Scheme(reconstruction="PPMC", riemann_solver="HLLC", dual_energy=True, precision=precision))
    Ua = cuda.from_numpy(U0.copy()).cuda()
    Us = cuda.from_numpy(U0.copy()).cuda()
    dts = []
    for _ in range(2):  # the allocating entry point first: its first call allocates its own scratch
        dt = 0.3 / I.Calc_dt_GPU(Ua, N, N, N, ng, nf, dx, dx, dx, 5 / 3)
        I.VL_Algorithm_3D_CUDA(Ua, None, N, N, N, 0, 0, 0, ng, dx, dx, dx, 0, 0, 0, dt, nf, 0, 0.0)
        I.Set_Boundaries(Ua, N, N, N, ng, nf, (1,) * 6)
        dts.append(dt)
    # first static call on this device: it looks up the pool, and under lazy module loading the
    # driver maps the module's static data (the 24 MiB pool) at that moment
    Uw = cuda.from_numpy(U0.copy()).cuda()
    assert _static_step(lib, Uw, N, ng, dx, dts[0], nf) == _lib.CGB_OK, lib.cgb_last_error().decode()
    cuda.cuda.synchronize()
    free_before = cuda.cuda.mem_get_info()[0]
    for dt in dts:  # two calls in a row through the static pool, same dt sequence
        rc = _static_step(lib, Us, N, ng, dx, dt, nf)
        assert rc == _lib.CGB_OK, lib.cgb_last_error().decode()
        I.Set_Boundaries(Us, N, N, N, ng, nf, (1,) * 6)
    cuda.cuda.synchronize()
    assert cuda.cuda.mem_get_info()[0] == free_before, "device free memory changed across the static calls"
    rs = real_slice(ng)
    a, s = Ua.cpu().numpy()[rs], Us.cpu().numpy()[rs]
    assert np.isfinite(s).all()
    err = np.abs(s - a).sum(axis=(1, 2, 3)) / np.abs(a).sum(axis=(1, 2, 3))
    assert np.all(err <= PRECISIONS[precision]), err


@pytest.mark.parametrize("precision,n", [("fp64", 80), ("fp64_fast", 64)])
def test_static_step_rejects_box_larger_than_pool(cuda, precision, n):
    from cholla_gb300 import _lib
    from cholla_gb300 import integrator as I

    lib = _lib.lib()
    ng, nf = 4, 6
    N = n + 2 * ng
    I.set_scheme(I.Scheme(reconstruction="PPMC", riemann_solver="HLLC", dual_energy=True, precision=precision))
    U = cuda.zeros(8, dtype=cuda.float64, device="cuda")  # never touched: the size check comes first
    rc = _static_step(lib, U, N, ng, 1 / n, 1e-3, nf)
    assert rc == _lib.CGB_ERR_ARGS
    msg = lib.cgb_last_error().decode()
    assert "static pool" in msg and "bytes" in msg, msg
    I.set_scheme(I.Scheme())


@pytest.mark.parametrize("precision,N", [("fp64", 73), ("fp64_fast", 58), ("mixed", 58)])
def test_static_step_accepts_largest_box(cuda, precision, N):
    """The largest cube the pool holds with 6 fields: 73^3 padded cells in FP64 ((f + 2) 8 n bytes),
    58^3 in the fast forms ((2 f + 4) 8 n bytes), each plus 512 bytes and array rounding."""
    from cholla_gb300 import _lib, ics
    from cholla_gb300 import integrator as I

    lib = _lib.lib()
    ng = 4
    n = N - 2 * ng
    U0 = ics.turbulence_box(n, ng, 5 / 3, seed=9)
    nf = U0.shape[0]
    I.set_scheme(I.Scheme(reconstruction="PPMC", riemann_solver="HLLC", dual_energy=True, precision=precision))
    U = cuda.from_numpy(U0.copy()).cuda()
    dt = 0.3 / I.Calc_dt_GPU(U, N, N, N, ng, nf, 1 / n, 1 / n, 1 / n, 5 / 3)
    rc = _static_step(lib, U, N, ng, 1 / n, dt, nf)
    assert rc == _lib.CGB_OK, lib.cgb_last_error().decode()
    cuda.cuda.synchronize()
    assert np.isfinite(U.cpu().numpy()[real_slice(ng)]).all()
    I.set_scheme(I.Scheme())
