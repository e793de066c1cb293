import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (REPO, os.path.join(REPO, "glsl-tree-construction_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); parity of the CUDA path against the oracle")
    config.addinivalue_line("markers", "slow: full-size workload")


@pytest.fixture(scope="session")
def oracle():
    import oracle as O

    O.build()
    return O


@pytest.fixture(scope="session")
def gtc_mod():
    import gtc

    gtc.lib()  # fails loudly if libgtc.so is missing
    return gtc


@pytest.fixture(scope="session")
def ctx(gtc_mod):
    import torch

    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    c = gtc_mod.Context(0)
    yield c
    c.close()
