"""Initial conditions on the host: the random fields follow the stated shell spectrum, the
turbulence box has the stated statistics, and the blast box deposits the stated energy; the
accuracy report refuses an unknown FP64 baseline."""
import math

import numpy as np
import pytest

from cholla_gb300 import ics


def _shell_spectrum_slope(f):
    n = f.shape[0]
    k = np.fft.fftfreq(n) * n
    kk = np.sqrt(k[:, None, None] ** 2 + k[None, :, None] ** 2 + k[None, None, :] ** 2)
    p = np.abs(np.fft.fftn(f)) ** 2
    kb = np.arange(2, n // 4)
    e = np.array([p[(kk >= a - 0.5) & (kk < a + 0.5)].sum() for a in kb])  # E(k) dk, summed over the shell
    return np.polyfit(np.log(kb), np.log(e), 1)[0]


def test_random_field_has_the_stated_shell_spectrum():
    rng = np.random.default_rng(0)
    for slope in (-2.0, -3.0):
        f = ics.gaussian_random_field(64, slope, rng)
        assert abs(f.mean()) < 1e-12 and abs(f.std() - 1.0) < 1e-12
        assert abs(_shell_spectrum_slope(f) - slope) < 0.15


def test_turbulence_box_statistics():
    n, ng, gamma, mach = 32, 4, 5 / 3, 2.0
    U = ics.turbulence_box(n, ng, gamma, seed=3, mach=mach)
    r = U[:, ng:-ng, ng:-ng, ng:-ng]
    rho = r[0]
    assert abs(rho.mean() - 1.0) < 0.05 and abs(np.log(rho).std() - 0.5) < 0.01
    v2 = ((r[1:4] / rho) ** 2).sum(axis=0)
    assert abs(math.sqrt(v2.mean()) - mach * math.sqrt(gamma)) < 1e-9  # rms Mach 2 at p = rho = 1
    eint = r[4] - 0.5 * rho * v2
    assert np.allclose(eint, 1.0 / (gamma - 1.0)) and np.allclose(r[5], eint)  # uniform pressure, GasEnergy
    assert np.array_equal(U[:, :ng], U[:, n:n + ng])  # periodic ghost layers


def test_blast_box_deposits_the_energy():
    n, ng, gamma = 24, 4, 5 / 3
    U = ics.blast_box(n, ng, gamma, energy=1.0, p=1e-5)
    r = U[:, ng:-ng, ng:-ng, ng:-ng]
    excess = (r[4] - 1e-5 / (gamma - 1.0)).sum() / n ** 3
    assert abs(excess - 1.0) < 1e-12 and np.all(r[1:4] == 0) and np.all(r[0] == 1.0)


def test_accuracy_run_rejects_an_unknown_baseline():
    """The accuracy report's FP64 baseline is the exact or the fast FP64 form; anything else is
    refused before any device work."""
    import torch

    from cholla_gb300 import accuracy

    with pytest.raises(ValueError):
        accuracy.run(torch, n=8, steps=1, baseline="mixed")
