"""The mixed form's integer-pipe binary64 <-> binary32 conversions equal the hardware
conversions bit for bit: random bit
patterns over every exponent, the halfway and carry cases of rounding to nearest even, the edges
of the binary32 normal range, results on the binary32 subnormal grid, zeros, subnormal inputs,
infinities; a NaN has to give a NaN (its payload is not compared)."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _patterns():
    rng = np.random.default_rng(11)
    bits = [rng.integers(0, 2 ** 63, size=1 << 20, dtype=np.int64).view(np.uint64),
            rng.integers(0, 2 ** 63, size=1 << 20, dtype=np.int64).view(np.uint64) | np.uint64(1 << 63)]
    # exponents around the binary32 range, with fractions at and beside the rounding point
    e = np.arange(850, 1200, dtype=np.uint64)  # 850 .. 896: the binary32 subnormal range and below
    frac = np.array([0, 1, (1 << 28) - 1, 1 << 28, (1 << 28) + 1, (1 << 29), (1 << 29) | (1 << 28),
                     (1 << 52) - 1, (1 << 52) - (1 << 28), ((1 << 52) - 1) ^ ((1 << 29) - 1)], dtype=np.uint64)
    grid = (e[:, None] << np.uint64(52)) | frac[None, :]
    bits += [grid.ravel(), grid.ravel() | np.uint64(1 << 63)]
    specials = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 1e-40, -1e-40, 3.4028234663852886e38,
                         3.4028235677973366e38, 1.1754943508222875e-38, 1.1754942807573643e-38, 1.0, 1.5],
                        dtype=np.float64).view(np.uint64)
    bits.append(specials)
    # results on the binary32 subnormal grid (exponent fields 873 .. 896, units of 2^-149 = the
    # 53-bit significand S >> (926 - e)): halfway cases with an even and an odd kept part, and
    # one unit either side of halfway
    sub = []
    for ex in range(873, 897):
        sh = 926 - ex
        qs = (0,) if sh >= 53 else (1 << (52 - sh), (1 << (52 - sh)) + 1, (1 << (53 - sh)) - 1)
        for q in qs:
            for rem in ((1 << (sh - 1)), (1 << (sh - 1)) - 1, (1 << (sh - 1)) + 1):
                S = (q << sh) | rem
                if (1 << 52) <= S < (1 << 53):
                    sub.append((ex << 52) | (S - (1 << 52)))
    sub = np.array(sub, dtype=np.uint64)
    bits += [sub, sub | np.uint64(1 << 63)]
    # the binary32 read from each low word: make some low words normal floats, halfway values etc.
    f32 = rng.integers(0, 2 ** 32, size=1 << 16, dtype=np.uint64)
    f32 = np.concatenate([f32, np.array([0, 0x80000000, 1, 0x80000001, 0x007fffff, 0x807fffff, 0x00400000,
                                         0x7f800000, 0xff800000, 0x7fc00000, 0x7f800001, 0x00800000],
                                        dtype=np.uint64)])
    bits.append((np.uint64(0x3ff) << np.uint64(52)) | f32)
    return np.concatenate(bits).view(np.float64)


def test_integer_pipe_conversions_match_hardware(cuda):
    from cholla_gb300 import _lib as L

    x = cuda.from_numpy(_patterns()).cuda()
    bad = (C.c_ulonglong * 2)()
    rc = L.lib().cgb_selftest_conversions(C.c_void_p(x.data_ptr()), x.numel(), bad, None)
    assert rc == L.CGB_OK
    assert bad[0] == 0 and bad[1] == 0, (bad[0], bad[1])
