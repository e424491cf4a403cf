import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle

    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def ref_host(oracle_lib):
    """The reference's own VL integrators compiled as host code (oracle/build_ref_host.sh), built
    on first use where the reference source tree is present; the tests that need it skip
    elsewhere."""
    import subprocess

    from oracle import ref_host

    tree = Path(os.environ.get("CHOLLA_REFERENCE", ROOT.parent / "reference"))
    if tree.is_dir():
        subprocess.run(["bash", str(ROOT / "oracle" / "build_ref_host.sh"), str(tree)], check=True,
                       stdout=subprocess.DEVNULL)
    if not ref_host.available("ppmc_hllc_de"):
        pytest.skip("the reference source tree is absent: no host-compiled reference")
    return ref_host


@pytest.fixture(scope="session")
def cuda():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch
