"""The batch C ABI and the autotuner's host side without a GPU: a batch refuses schemes and
arguments it cannot run before it touches the device, calls on a null handle fail cleanly,
and the tuner's cache key depends on the size mix (not its order) and on the scheme."""
import ctypes as C

import pytest


@pytest.fixture(scope="module")
def lib():
    from cholla_gb300 import _lib

    return _lib.lib()


def _create(lib, scheme, c_cfl=0.3, stream=0x10):
    h = C.c_void_p()
    s = scheme.to_c()
    rc = lib.cgb_batch_create(C.byref(h), C.byref(s), c_cfl, C.c_void_p(stream))
    return rc, h


def test_batch_create_refuses_what_it_cannot_run(lib):
    from cholla_gb300 import _lib
    from cholla_gb300 import integrator as I

    mixed = I.Scheme(reconstruction="PPMC", riemann_solver="HLLC", dual_energy=True, precision="mixed")
    cases = [
        (I.Scheme(riemann_solver="HLLD", mhd=True, dual_energy=False), 0.3, 0x10, _lib.CGB_ERR_UNSUPPORTED),
        (I.Scheme(precision="fp64"), 0.3, 0x10, _lib.CGB_ERR_UNSUPPORTED),  # exact form: single boxes only
        (mixed, 0.0, 0x10, _lib.CGB_ERR_ARGS),                               # CFL number must be positive
        (mixed, 0.3, 0, _lib.CGB_ERR_ARGS),                                  # a batch needs its own stream
    ]
    for scheme, c_cfl, stream, code in cases:
        rc, h = _create(lib, scheme, c_cfl, stream)
        assert rc == code, (scheme, c_cfl, stream, rc)
        assert not h.value
        assert lib.cgb_batch_last_error()


def test_batch_calls_on_a_null_handle_fail_cleanly(lib):
    from cholla_gb300 import _lib

    null = C.c_void_p()
    t, dt = C.c_double(), C.c_double()
    assert lib.cgb_batch_step(null, 1) == _lib.CGB_ERR_ARGS
    assert lib.cgb_batch_remove(null, 1) == _lib.CGB_ERR_ARGS
    assert lib.cgb_batch_hold(null, 1, 1) == _lib.CGB_ERR_ARGS
    assert lib.cgb_batch_set_chains(null, 2) == _lib.CGB_ERR_ARGS
    assert lib.cgb_batch_set_solo_cells(null, 1 << 20) == _lib.CGB_ERR_ARGS
    assert lib.cgb_batch_set_tiles(null, 1) == _lib.CGB_ERR_ARGS
    assert lib.cgb_batch_job_time(null, 1, C.byref(t), C.byref(dt)) == _lib.CGB_ERR_ARGS
    assert lib.cgb_batch_n_jobs(null) == -1
    assert lib.cgb_batch_destroy(null) == _lib.CGB_OK


def test_tuner_cache_key():
    from cholla_gb300 import tune
    from cholla_gb300.serve import default_scheme

    s = default_scheme()
    assert tune._key([32, 64, 32], s) == tune._key([64, 32, 32], s)
    assert tune._key([32, 64], s) != tune._key([32, 64, 64], s)
    f = default_scheme()
    f.precision = "fp64_fast"
    assert tune._key([32, 64], s) != tune._key([32, 64], f)
