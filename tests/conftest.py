import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "bacterial-classification_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def orc():
    from oracle import oracle
    oracle.lib()
    return oracle


@pytest.fixture(scope="session")
def hdc():
    """The built C-ABI library (built on first use, as __graft_entry__.build() does)."""
    import build as pkg_build
    pkg_build.build()
    import hdc_gb300
    hdc_gb300.lib()
    return hdc_gb300


@pytest.fixture(scope="session")
def cuda(hdc):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda:0")
