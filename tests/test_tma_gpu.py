"""The TMA staging of the fast forms' corrector sweeps.

* Staged by the Tensor Memory Accelerator or loaded thread by thread, two steps give the same
  state to rounding (fast FP64 and mixed precision, PPMC / PLMC / PCM, with dual energy and scalars,
  on a box whose real extent is not a multiple of the tile, so partial tiles read past the array).
  The two are separate kernels, and the code generator contracts multiplies and adds into FMAs
  kernel by kernel, so a few values may differ in the last bits (mostly they agree bit for bit);
  a wrong tile would show as an O(1) error in its cells.  Bars: relative L1 per field 1e-7 (mixed)
  / 1e-14 (fast FP64), and the largest difference per field within 1e-5 (mixed) / 1e-11 (fast
  FP64) of the field's largest value.  Each form repeats itself bit for bit.
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
        for tma in (1, 0, 1):
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
    a, b, a2 = out[0][rs], out[1][rs], out[2][rs]
    assert np.isfinite(a).all()
    assert np.array_equal(a.view(np.int64), a2.view(np.int64))
    l1_bar, max_bar = (1e-7, 1e-5) if precision == "mixed" else (1e-14, 1e-11)
    l1 = np.abs(a - b).sum(axis=(1, 2, 3)) / np.abs(b).sum(axis=(1, 2, 3))
    worst = np.max(np.abs(a - b).max(axis=(1, 2, 3)) / np.abs(b).max(axis=(1, 2, 3)))
    print(f"{precision} {recon}: {(a != b).sum()} of {a.size} values differ; rel L1 {l1.max():.2e}, max rel {worst:.2e}")
    assert np.all(l1 <= l1_bar), l1
    assert worst <= max_bar, worst


def test_bounded_wait_reports_timeout(cuda):
    from cholla_gb300 import _lib as L

    st = cuda.zeros(1, dtype=cuda.int32, device="cuda")
    rc = L.lib().cgb_selftest_tma_timeout(ctypes.c_void_p(st.data_ptr()), 2000, None)
    assert rc == L.CGB_OK
    assert int(st.item()) & L.CGB_STATUS_TIMEOUT
