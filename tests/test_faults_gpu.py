"""Failure reporting, with every failure made on the host.

* A corrupted request (NaN, or a negative density, written into the host state before upload)
  is reported as CGB_ERR_NONFINITE by the box engine, the batch (for that job only: the other
  jobs' results are unchanged bit for bit) and the drop-in entry points (cgb_check_status), as
  the reference reports crashed cells from the device (src/hydro/hydro_cuda.cu:381-389).
* A device allocation failure, injected on the host through cgb_debug_fail_alloc, turns into
  CGB_ERR_NOMEM at every allocating entry point, leaks nothing, and the next call succeeds.
* The MHD divergence check of src/mhd/magnetic_divergence.cu:92-120 rejects a field whose
  divergence exceeds 1e-9.

Nothing here faults, traps or hangs the GPU: the bad values are ordinary IEEE doubles and the
allocation failure never reaches CUDA.
"""
import numpy as np
import pytest

from helpers import real_slice

pytestmark = pytest.mark.gpu

NG = 4


def _scheme(precision="mixed"):
    from cholla_gb300 import integrator as I

    return I.Scheme(reconstruction="PPMC", riemann_solver="HLLC", dual_energy=True, density_floor=True,
                    temperature_floor=True, precision=precision)


def _corrupt(U0, how):
    U = U0.copy()
    c = (NG + 3, NG + 5, NG + 2)
    if how == "nan":
        U[(0, *c)] = np.nan
    else:  # a negative density and an energy that cannot go with it
        U[(0, *c)] = -1.0
    return U


@pytest.mark.parametrize("precision", ["fp64", "fp64_fast", "mixed"])
@pytest.mark.parametrize("how", ["nan", "negative"])
def test_box_reports_corrupted_state(cuda, precision, how):
    from cholla_gb300 import _lib as L
    from cholla_gb300 import ics
    from cholla_gb300.engine import Box, BoxError

    n = 16
    U0 = ics.turbulence_box(n, NG, 5 / 3, seed=3)
    N = n + 2 * NG
    good = Box(N, N, N, NG, 1 / n, 1 / n, 1 / n, _scheme(precision))
    Ug = cuda.from_numpy(U0.copy()).cuda()
    good.advance(Ug, 3, 0.3)
    good.time()  # no error on a clean state
    assert good.check_status() & L.CGB_STATUS_NONFINITE == 0
    box = Box(N, N, N, NG, 1 / n, 1 / n, 1 / n, _scheme(precision))
    Ub = cuda.from_numpy(_corrupt(U0, how)).cuda()
    box.advance(Ub, 2, 0.3)
    with pytest.raises(BoxError) as e:
        box.time()
    assert e.value.code == L.CGB_ERR_NONFINITE
    with pytest.raises(BoxError):
        box.check_status()
    box.close()
    good.close()


def test_batch_reports_only_the_corrupted_job(cuda):
    from cholla_gb300 import _lib as L
    from cholla_gb300 import ics
    from cholla_gb300.batch import Batch, BatchError

    stream = cuda.cuda.Stream()
    scheme = _scheme("mixed")
    states = [ics.turbulence_box(n, NG, 5 / 3, seed=10 + n) for n in (16, 24, 20)]

    def run(corrupt_middle):
        b = Batch(scheme, stream)
        Us, ids = [], []
        for i, U0 in enumerate(states):
            U = _corrupt(U0, "nan") if (corrupt_middle and i == 1) else U0.copy()
            Ug = cuda.from_numpy(U).cuda()
            n = U0.shape[1] - 2 * NG
            ids.append(b.add(Ug, NG, 1 / n, 1 / n, 1 / n))
            Us.append(Ug)
        b.step(4)
        codes = []
        for j in ids:
            try:
                b.job_time(j)
                codes.append(L.CGB_OK)
            except BatchError as ex:
                codes.append(ex.code)
        flags = [b.job_status(j) for j in ids]
        out = [U.cpu().numpy() for U in Us]
        b.close()
        return codes, flags, out

    codes_ok, flags_ok, clean = run(False)
    assert codes_ok == [L.CGB_OK] * 3 and all(f & L.CGB_STATUS_NONFINITE == 0 for f in flags_ok)
    codes, flags, mixed = run(True)
    assert codes == [L.CGB_OK, L.CGB_ERR_NONFINITE, L.CGB_OK]
    assert flags[1] & L.CGB_STATUS_NONFINITE
    for i in (0, 2):  # the healthy jobs are unaffected, bit for bit
        assert np.array_equal(mixed[i].view(np.int64), clean[i].view(np.int64))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_dropin_check_status(cuda, precision):
    from cholla_gb300 import _lib as L
    from cholla_gb300 import ics
    from cholla_gb300 import integrator as I

    n = 16
    N, dx = n + 2 * NG, 1 / n
    U0 = ics.turbulence_box(n, NG, 5 / 3, seed=4)
    nf = U0.shape[0]
    I.set_scheme(_scheme(precision))
    I.Check_Status()  # clear whatever earlier calls left
    Ug = cuda.from_numpy(U0.copy()).cuda()
    dt = 0.3 / I.Calc_dt_GPU(Ug, N, N, N, NG, nf, dx, dx, dx, 5 / 3)
    I.VL_Algorithm_3D_CUDA(Ug, None, N, N, N, 0, 0, 0, NG, dx, dx, dx, 0, 0, 0, dt, nf, 0, 0.0)
    assert I.Check_Status() & L.CGB_STATUS_NONFINITE == 0
    Ub = cuda.from_numpy(_corrupt(U0, "nan")).cuda()
    I.VL_Algorithm_3D_CUDA(Ub, None, N, N, N, 0, 0, 0, NG, dx, dx, dx, 0, 0, 0, dt, nf, 0, 0.0)
    with pytest.raises(L.CgbError) as e:
        I.Check_Status()
    assert e.value.code == L.CGB_ERR_NONFINITE
    assert I.Check_Status() == 0  # the report cleared the word
    I.set_scheme(I.Scheme())


def test_injected_allocation_failures(cuda):
    """Every device allocation of box creation, a batch join and the drop-in scratch fails in turn;
    each failure is CGB_ERR_NOMEM, frees what the call had taken, and the call then succeeds."""
    from cholla_gb300 import _lib as L
    from cholla_gb300 import ics
    from cholla_gb300 import integrator as I
    from cholla_gb300.batch import Batch, BatchError
    from cholla_gb300.engine import Box, BoxError

    n = 16
    N, dx = n + 2 * NG, 1 / n
    U0 = ics.turbulence_box(n, NG, 5 / 3, seed=5)
    nf = U0.shape[0]
    cuda.cuda.synchronize()
    try:
        # box creation makes several allocations: fail each in turn
        free0 = cuda.cuda.mem_get_info()[0]
        for k in range(1, 16):
            I.debug_fail_alloc(k)
            try:
                b = Box(N, N, N, NG, dx, dx, dx, _scheme("fp64_fast"))
                b.close()
                I.debug_fail_alloc(0)
                break  # k is past the last allocation: creation succeeded
            except BoxError as e:
                assert e.code == L.CGB_ERR_NOMEM
        else:
            pytest.fail("box creation never completed")
        assert k > 1, "box creation made no allocation through the library's allocator"
        cuda.cuda.synchronize()
        assert cuda.cuda.mem_get_info()[0] >= free0 - (2 << 20)  # nothing leaked beyond allocator slack

        # batch join
        stream = cuda.cuda.Stream()
        bt = Batch(_scheme("mixed"), stream)
        Ua = cuda.from_numpy(U0.copy()).cuda()
        ja = bt.add(Ua, NG, dx, dx, dx)
        I.debug_fail_alloc(1)
        Ub = cuda.from_numpy(U0.copy()).cuda()
        with pytest.raises(BatchError) as e:
            bt.add(Ub, NG, dx, dx, dx)
        assert e.value.code == L.CGB_ERR_NOMEM
        assert len(bt) == 1
        bt.step(2)  # the batch still runs its job
        assert bt.job_time(ja)[0] > 0
        jb = bt.add(Ub, NG, dx, dx, dx)  # and the join succeeds once memory is there
        bt.step(1)
        assert bt.job_time(jb)[0] > 0
        bt.close()

        # drop-in scratch (first call for a new shape allocates)
        I.Free_Memory_VL_3D()
        I.set_scheme(_scheme("fp64"))
        Ug = cuda.from_numpy(U0.copy()).cuda()
        I.debug_fail_alloc(1)
        with pytest.raises(L.CgbError) as e:
            I.VL_Algorithm_3D_CUDA(Ug, None, N, N, N, 0, 0, 0, NG, dx, dx, dx, 0, 0, 0, 1e-4, nf, 0, 0.0)
        assert e.value.code == L.CGB_ERR_NOMEM
        I.VL_Algorithm_3D_CUDA(Ug, None, N, N, N, 0, 0, 0, NG, dx, dx, dx, 0, 0, 0, 1e-4, nf, 0, 0.0)
        cuda.cuda.synchronize()
        assert np.isfinite(Ug.cpu().numpy()[real_slice(NG)]).all()
    finally:
        I.debug_fail_alloc(0)
        I.set_scheme(I.Scheme())


def test_magnetic_divergence_check(cuda):
    from cholla_gb300 import _lib as L
    from cholla_gb300 import ics
    from cholla_gb300 import integrator as I

    n, gamma = 16, 5 / 3
    s = I.Scheme(reconstruction="PLMC", riemann_solver="HLLD", mhd=True, dual_energy=False, gamma=gamma)
    ng = s.n_ghost()
    U0 = ics.mhd_box(n, ng, gamma, seed=2)
    nf, N = U0.shape[0], U0.shape[1]
    dx = 1 / n
    I.set_scheme(s)
    try:
        Ug = cuda.from_numpy(U0.copy()).cuda()
        I.Set_Boundaries(Ug, N, N, N, ng, nf, (1,) * 6)
        assert I.Check_Magnetic_Divergence(Ug, N, N, N, ng, nf, dx, dx, dx) <= L.CGB_MAX_DIVB
        Ub = U0.copy()
        Ub[5, ng + 4, ng + 4, ng + 4] += 1e-3  # one face field off: div B ~ 1e-3 / dx in two cells
        Ubg = cuda.from_numpy(Ub).cuda()
        I.Set_Boundaries(Ubg, N, N, N, ng, nf, (1,) * 6)
        with pytest.raises(L.CgbError) as e:
            I.Check_Magnetic_Divergence(Ubg, N, N, N, ng, nf, dx, dx, dx)
        assert e.value.code == L.CGB_ERR_NONFINITE
    finally:
        I.set_scheme(I.Scheme())
