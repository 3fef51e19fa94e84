import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle_py as O
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)
    return O


@pytest.fixture(scope="session")
def valib():
    """The CUDA library, built in-tree if needed (nvcc cross-compiles without a GPU)."""
    from vectorizedadjoint_gb300 import build as vbuild
    vbuild.build()
    import vectorizedadjoint_gb300 as va
    return va


@pytest.fixture(scope="session")
def cuda(valib):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.set_device(0)
    return torch
