"""The TMA staging of the fast forms' corrector sweeps.

* Staged by the Tensor Memory Accelerator or loaded thread by thread, a step gives the same state
  bit for bit (fast FP64 and mixed precision, PPMC / PLMC / PCM, with dual energy and scalars, on a
  box whose real extent is not a multiple of the tile, so partial tiles read past the array).
* The bounded mbarrier wait gives up when the bytes it expects never arrive and reports
  CGB_STATUS_TIMEOUT: the self-test's mbarrier expects bytes that no copy delivers (no copy is
  issued, so nothing is left in flight and nothing faults).
"""
import ctypes

import numpy as np
import pytest

from helpers import real_slice

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp64_fast", "mixed"])
@pytest.mark.parametrize("recon,ns", [("PPMC", 0), ("PLMC", 1), ("PCM", 0)])
def test_tma_staging_equals_plain_loads(cuda, precision, recon, ns):
    from cholla_gb300 import _lib as L
    from cholla_gb300 import ics
    from cholla_gb300 import integrator as I

    ng = {"PCM": 2, "PLMC": 3, "PPMC": 4}[recon]
    rng = np.random.default_rng(77)
    U0 = ics.smooth_random_box((70, 37, 44), ng, rng, dual_energy=True, n_scalars=ns)
    nf, nz, ny, nx = U0.shape
    dx = (1 / 70, 1 / 37, 1 / 44)
    dt = 0.2 * min(dx)
    I.set_scheme(I.Scheme(reconstruction=recon, dual_energy=True, n_scalars=ns, precision=precision))
    out = []
    try:
        for tma in (1, 0):
            assert L.lib().cgb_set_tma(tma) == L.CGB_OK
            U = cuda.from_numpy(U0.copy()).cuda()
            for _ in range(2):
                I.VL_Algorithm_3D_CUDA(U, None, nx, ny, nz, 0, 0, 0, ng, *dx, 0, 0, 0, dt, nf, 0, 0.0)
                I.Set_Boundaries(U, nx, ny, nz, ng, nf, (1,) * 6)
            assert I.Check_Status() & L.CGB_STATUS_TIMEOUT == 0
            out.append(U.cpu().numpy())
    finally:
        L.lib().cgb_set_tma(1)
        I.set_scheme(I.Scheme())
    rs = real_slice(ng)
    a, b = out[0][rs], out[1][rs]
    assert np.isfinite(a).all()
    assert np.array_equal(a.view(np.int64), b.view(np.int64)), f"{(a != b).sum()} values differ"


def test_bounded_wait_reports_timeout(cuda):
    from cholla_gb300 import _lib as L

    st = cuda.zeros(1, dtype=cuda.int32, device="cuda")
    rc = L.lib().cgb_selftest_tma_timeout(ctypes.c_void_p(st.data_ptr()), 2000, None)
    assert rc == L.CGB_OK
    assert int(st.item()) & L.CGB_STATUS_TIMEOUT
