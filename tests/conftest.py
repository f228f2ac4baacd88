import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    import oracle as O
    O.build(ref=True)
    return O


@pytest.fixture(scope="session")
def tsim():
    """The CUDA library, built for sm_103a (fails loudly if it cannot be)."""
    import cudaruntime1_gb300 as T
    T.build()
    return T


@pytest.fixture(scope="session")
def cuda_ctx(tsim):
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test run without a CUDA device")
    ctx = tsim.Context(0)
    yield ctx
    ctx.close()
