"""The throughput forms against the exact FP64 form on the same dt sequence (the accuracy
report run at a small size): mixed precision within 1e-5 relative L1 in density, the fast
FP64 form at rounding level; mass and momenta of a periodic box that never reaches the
density floor are conserved to accumulation roundoff by every form."""
import pytest

pytestmark = pytest.mark.gpu


def test_accuracy_report_small_box(cuda):
    from cholla_gb300 import accuracy

    r = accuracy.run(cuda, n=32, steps=8, seed=3)  # rms Mach 2
    assert r["rel_l1"]["mixed"]["density"] <= 1e-5, r["rel_l1"]["mixed"]
    assert max(r["rel_l1"]["mixed"].values()) <= 1e-4, r["rel_l1"]["mixed"]
    assert max(r["rel_l1"]["fp64_fast"].values()) <= 1e-11, r["rel_l1"]["fp64_fast"]
    for form, c in r["conservation"].items():
        assert c["momentum"] <= 1e-13, (form, c)


def test_conservation_without_floor_events(cuda):
    from cholla_gb300 import accuracy

    r = accuracy.run(cuda, n=32, steps=8, seed=3, mach=0.5)
    for form, c in r["conservation"].items():
        assert c["mass"] <= 1e-13 and c["momentum"] <= 1e-13, (form, c)
