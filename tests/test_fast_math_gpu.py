"""Error of the fast FP64 form's reciprocal and square root (cholla_gb300/csrc/hydro_fast.cuh:
rcp, an FP32 estimate and one third-order iteration r (1 + e + e^2); sqrtT, one Newton-Raphson
step on the inverse square root and the Karp-Markstein correction) against CUDA's correctly rounded 1 / x and
sqrt, measured in units in the last place over the FP32 exponent range and on both sides of the
2^-99 / 2^99 guards, where the helpers switch to the true divide and square root."""
import numpy as np
import pytest

from helpers import ulp_diff

pytestmark = pytest.mark.gpu

MAX_ULP = 1  # the bound the helpers' comment states


def _inputs():
    rng = np.random.default_rng(2024)
    mag = 10.0 ** rng.uniform(-38, 38, 400_000)  # beyond the guards on both sides
    x = mag * np.where(rng.random(mag.size) < 0.5, -1.0, 1.0)
    edges = []
    for e in (1e-30, 1e30, 1.0, 2.0, 0.5, np.float64(np.float32(1e-30)), np.float64(np.float32(1e30)),
              np.ldexp(1.0, -99), np.ldexp(1.0, 99)):
        edges += list(np.nextafter(e, 0) * np.array([1.0, -1.0])) + [e, -e] + list(np.nextafter(e, np.inf) *
                                                                                np.array([1.0, -1.0]))
        edges += list(e * (1 + np.arange(-40, 41) * 2.0 ** -30))
    edges += list(np.float64(np.float32(rng.uniform(1, 2, 20_000))))  # binary32-representable inputs
    return np.concatenate([x, np.array(edges, dtype=np.float64)])


def test_rcp_and_sqrt_within_one_ulp(cuda):
    import ctypes

    from cholla_gb300 import _lib as L

    x = _inputs()
    n = x.size
    d_x = cuda.from_numpy(x).cuda()
    d_out = cuda.empty(4 * n, dtype=cuda.float64, device="cuda")
    rc = L.lib().cgb_selftest_fast_math(ctypes.c_void_p(d_x.data_ptr()), n, ctypes.c_void_p(d_out.data_ptr()), None)
    assert rc == L.CGB_OK
    out = d_out.cpu().numpy().reshape(4, n)
    fast_rcp, cuda_rcp, fast_sqrt, cuda_sqrt = out
    # CUDA's __drcp_rn and __dsqrt_rn are IEEE correctly rounded: numpy's must agree bit for bit
    assert np.array_equal(cuda_rcp.view(np.int64), (1.0 / x).view(np.int64))
    assert np.array_equal(cuda_sqrt.view(np.int64), np.sqrt(np.abs(x)).view(np.int64))
    u_rcp = ulp_diff(fast_rcp, cuda_rcp)
    u_sqrt = ulp_diff(fast_sqrt, cuda_sqrt)
    frac_r = float(np.mean(u_rcp == 0))
    frac_s = float(np.mean(u_sqrt == 0))
    assert u_rcp.max() <= MAX_ULP, (u_rcp.max(), x[np.argmax(u_rcp)], frac_r)
    assert u_sqrt.max() <= MAX_ULP, (u_sqrt.max(), x[np.argmax(u_sqrt)], frac_s)
    print(f"rcp: max {u_rcp.max()} ulp, {frac_r:.4f} correctly rounded; "
          f"sqrt: max {u_sqrt.max()} ulp, {frac_s:.4f} correctly rounded")
